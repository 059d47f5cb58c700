// swgpu_api.cu -- the C ABI of libswgpu.so (declared in include/swgpu.h):
// device allocation and upload of a mesh, quantity transfer, the
// per-method entry points that mirror the reference's Domain overrides,
// and the device-resident evolve loop (CUDA graphs of several Euler steps,
// host synchronisation only between graphs).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "swgpu_handle.cuh"

namespace swgpu {

static thread_local std::string g_create_error;

// Message for swgpu_last_error(NULL) from entry points that have no handle.
void record_global_error(const char *message) { g_create_error = message; }

static int fail(Handle *h, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h)
        h->err = buf;
    else
        g_create_error = buf;
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(h, e_ == cudaErrorMemoryAllocation ? SWGPU_ENOMEM : SWGPU_ECUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__,       \
                        __LINE__);                                                       \
    } while (0)

template <typename T>
static int dalloc(Handle *h, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc((void **)p, count * sizeof(T)));
    h->allocs.push_back((void *)*p);
    CK(cudaMemsetAsync(*p, 0, count * sizeof(T), h->stream));
    return SWGPU_OK;
}

template <typename T>
static int upload(Handle *h, T *dst, const T *src, size_t count) {
    if (count == 0) return SWGPU_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

template <typename T>
static int download(Handle *h, T *dst, const T *src, size_t count) {
    if (count == 0) return SWGPU_OK;
    CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

// AoS [3k+i] (or [6k+j]) host array -> planes [i*N+k]
template <typename T, typename U>
static std::vector<T> to_planes(const U *src, int64_t N, int width) {
    std::vector<T> out((size_t)N * width);
    for (int64_t k = 0; k < N; k++)
        for (int j = 0; j < width; j++) out[(size_t)j * N + k] = (T)src[k * width + j];
    return out;
}

static int check_launch(Handle *h, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return fail(h, SWGPU_ECUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return SWGPU_OK;
}

// A handle whose kernels reported SWGPU_ETIMEOUT (a bounded wait for a
// tile's bulk copies ran out twice) may have left copies in flight into the
// shared memory of blocks that have exited; nothing it computes afterwards
// can be trusted, so every later call that reaches the device fails and
// only swgpu_destroy remains.
static int check_usable(Handle *h) {
    if (h->unusable)
        return fail(h, SWGPU_ETIMEOUT,
                    "handle unusable: a bounded device-side wait ran out earlier (bulk copies "
                    "may still have been in flight); destroy the handle");
    return SWGPU_OK;
}

static int sync_ctrl(Handle *h) {
    if (int rc = check_usable(h)) return rc;
    CK(cudaMemcpyAsync(h->h_ctrl, h->d_ctrl, sizeof(Ctrl) * h->nscen, cudaMemcpyDeviceToHost,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

static int push_ctrl(Handle *h) {
    if (int rc = check_usable(h)) return rc;
    CK(cudaMemcpyAsync(h->d_ctrl, h->h_ctrl, sizeof(Ctrl) * h->nscen, cudaMemcpyHostToDevice,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

static const char *status_text(int s) {
    switch (s) {
        case SWGPU_OK: return "ok";
        case SWGPU_EINVAL: return "invalid argument";
        case SWGPU_ECUDA: return "CUDA error";
        case SWGPU_ENOMEM: return "out of device memory";
        case SWGPU_EDENOMINATOR: return "semi-implicit update denominator <= 0";
        case SWGPU_ESMALLSTEP: return "timestep below evolve_min_timestep even at first order";
        case SWGPU_ENONFINITE: return "non-finite value reached the flux timestep";
        case SWGPU_EBED: return "discontinuous elevation across an edge";
        case SWGPU_EBOUNDARY: return "unknown boundary type";
        case SWGPU_EOVERSHOOT: return "model time overshot finaltime";
        case SWGPU_EMESH: return "inconsistent mesh";
        case SWGPU_ETIMEOUT: return "a bounded device-side wait ran out";
        default: return "unknown status";
    }
}

// Device-side failures recorded in Ctrl.status become the call's status.
static int device_status(Handle *h) {
    if (int rc = check_usable(h)) return rc;
    for (int i = 0; i < h->nscen; i++) {
        if (h->h_ctrl[i].status != 0) {
            const int s = h->h_ctrl[i].status;
            if (s == SWGPU_ETIMEOUT) h->unusable = true;
            if (h->nscen > 1)
                return fail(h, s, "scenario %d: device reported: %s", i, status_text(s));
            return fail(h, s, "device reported: %s", status_text(s));
        }
    }
    return SWGPU_OK;
}

// Per-method calls that reduce one timestep over the whole mesh have no
// meaning for an ensemble of independent scenarios.
static int require_single(Handle *h, const char *what) {
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (h->nscen > 1)
        return fail(h, SWGPU_EINVAL, "%s: not available on an ensemble handle", what);
    return SWGPU_OK;
}

static void fill_state(const Ctrl *c, swgpu_state *s) {
    s->time = c->time;
    s->yieldtime = c->yieldtime;
    s->finaltime = c->finaltime;
    s->timestep = c->timestep;
    s->flux_timestep = c->flux_timestep;
    s->recorded_max_timestep = c->rec_max;
    s->recorded_min_timestep = c->rec_min;
    s->order = c->order;
    s->smallsteps = c->smallsteps;
    s->number_of_steps = c->steps_since_yield;
    s->total_steps = c->total_steps;
    s->stop_reason = c->stop_reason;
    s->status = c->status;
}

static void reset_ftmin(Ctrl *c, const DevParams &P) {
    double m = P.evolve_max_timestep;
    std::memcpy(&c->ftmin_bits, &m, sizeof m);
}

// ----------------------------------------------------------- step issue

// One stage of a fused step: flux -> update (with the stage's backup or
// saxpy and clock bookkeeping) -> distribute with boundary values.
static void issue_stage(Handle *h, const Stage &stg) {
    const int flux_flags = kFused | (stg.kind == kStageMid || stg.kind == kStageLast
                                         ? kNoTimestep : 0);
    const int update_flags = kFused | kFrictionInline | (h->S.hmax ? kTrack : 0);
    const int dist_flags = kFused | kWriteBoundary;
    if (h->precision == SWGPU_FP64) {
        launch_flux_fp64(h->M, h->S, h->P, h->d_ctrl, flux_flags, h->stream);
        launch_update_fp64(h->M, h->S, h->P, h->d_ctrl, 0.0, update_flags, stg, h->stream);
        launch_distribute_fp64(h->M, h->S, h->P, h->d_tags, h->d_ctrl, dist_flags, h->stream);
    } else {
        launch_flux_mixed(h->M, h->S, h->X, h->P, h->d_ctrl, flux_flags, h->stream);
        if (!(flux_flags & kNoTimestep))
            launch_step_clock_mixed(h->P, h->d_ctrl, h->nscen, h->M.shape.pdl, h->stream);
        launch_update_mixed(h->M, h->S, h->X, h->P, h->d_ctrl, update_flags, stg, h->stream);
        launch_distribute_mixed(h->M, h->S, h->X, h->P, h->d_tags, h->d_ctrl, dist_flags, stg,
                                h->stream);
    }
}

// The stages of one step of the handle's timestepping method (ANUGA's
// evolve_one_euler_step / evolve_one_rk2_step / evolve_one_rk3_step followed
// by the evolve loop's set_time, distribute and update_boundary).
static void issue_step(Handle *h) {
    if (h->timestepping_method == SWGPU_RK2) {
        issue_stage(h, Stage{kStageFirst, 1.0, 0.0, 1.0});
        issue_stage(h, Stage{kStageLast, 0.5, 0.5, 1.0});
    } else if (h->timestepping_method == SWGPU_RK3) {
        issue_stage(h, Stage{kStageFirst, 1.0, 0.0, 1.0});
        issue_stage(h, Stage{kStageMid, 0.25, 0.75, 0.5});
        issue_stage(h, Stage{kStageLast, 2.0 / 3.0, 1.0 / 3.0, 1.0});
    } else {
        issue_stage(h, kEulerStage);
    }
}

static int issue_fused_step(Handle *h) {
    issue_step(h);
    return check_launch(h, "evolve step");
}

// Captures `steps` fused steps into *exec (left as is when already built).
static int capture_steps(Handle *h, int steps, cudaGraphExec_t *exec) {
    if (*exec) return SWGPU_OK;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; s++) issue_step(h);
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return fail(h, SWGPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    return SWGPU_OK;
}

static int build_graph(Handle *h) { return capture_steps(h, h->steps_per_graph, &h->graph); }

// Drops the captured graphs after a change of what a step issues (launch
// shape, extent, stages, tracking); they are recaptured on the next run.
// The stream must be idle.
static void drop_graphs(Handle *h) {
    if (h->graph) cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
}

// distribute as the stand-alone method: protect + velocities, then the
// extrapolation/balance pass with edge values materialised.
static int issue_distribute(Handle *h, bool with_boundary) {
    if (h->precision == SWGPU_FP64) {
        launch_prepare_fp64(h->M, h->S, h->P, h->d_ctrl, h->stream);
        launch_distribute_fp64(h->M, h->S, h->P, h->d_tags, h->d_ctrl,
                               kWriteEdges | (with_boundary ? kWriteBoundary : 0), h->stream);
    } else {
        launch_prepare_mixed(h->M, h->S, h->X, h->P, h->mixed_from_stage ? 1 : 0, h->stream);
        h->mixed_from_stage = false;
        launch_distribute_mixed(h->M, h->S, h->X, h->P, h->d_tags, h->d_ctrl,
                                with_boundary ? kWriteBoundary : 0, kEulerStage, h->stream);
    }
    h->vertices_stale = false;
    return check_launch(h, "distribute");
}

}  // namespace swgpu

using namespace swgpu;

// ================================================================ C ABI ==

extern "C" {

const char *swgpu_last_error(void *handle) {
    if (!handle) return g_create_error.c_str();
    return static_cast<Handle *>(handle)->err.c_str();
}

int swgpu_device_info(char *buf, int buflen) {
    Handle *h = nullptr;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CK(cudaGetDeviceProperties(&p, dev));
    if (buf && buflen > 0)
        snprintf(buf, buflen, "%s sm_%d%d, %d SMs, %.1f GB (libswgpu %d)", p.name, p.major,
                 p.minor, p.multiProcessorCount, p.totalGlobalMem / 1e9, SWGPU_ABI_VERSION);
    return SWGPU_OK;
}

// Blocks of each scenario in one launch of each fused-step kernel (the
// last-block-done counts) for the handle's launch shape.
static void set_block_counts(Handle *h) {
    for (int i = 0; i < h->nscen; i++) {
        const int64_t n =
            h->nscen > 1 ? h->scen_offsets[i + 1] - h->scen_offsets[i] : (int64_t)h->M.N;
        Ctrl *c = &h->h_ctrl[i];
        c->blocks_flux = (unsigned)((n + h->M.shape.flux - 1) / h->M.shape.flux);
        c->blocks_update = (unsigned)((n + h->M.shape.update - 1) / h->M.shape.update);
        c->blocks_distribute =
            (unsigned)((n + h->M.shape.distribute - 1) / h->M.shape.distribute);
    }
}

// Shared by swgpu_create (offsets == nullptr, one scenario) and
// swgpu_create_ensemble.
static int create_impl(const swgpu_mesh *mesh, const swgpu_params *params, int precision,
                       const int64_t *offsets, int nscen, void **handle_out) {
    Handle *h = nullptr;
    if (!mesh || !params || !handle_out) return fail(nullptr, SWGPU_EINVAL, "null argument");
    *handle_out = nullptr;
    if (precision != SWGPU_FP64 && precision != SWGPU_MIXED)
        return fail(nullptr, SWGPU_EINVAL, "precision must be SWGPU_FP64 or SWGPU_MIXED");
    const int64_t N = mesh->number_of_elements, Nb = mesh->number_of_boundary_elements;
    if (N <= 0 || N >= (int64_t(1) << 29) || Nb < 0 || Nb > 3 * N)
        return fail(nullptr, SWGPU_EINVAL, "bad sizes N=%lld Nb=%lld", (long long)N,
                    (long long)Nb);
    if (!mesh->neighbours || !mesh->neighbour_edges || !mesh->surrogate_neighbours ||
        !mesh->number_of_boundaries || !mesh->normals || !mesh->edgelengths || !mesh->radii ||
        !mesh->areas || !mesh->vertex_coordinates || !mesh->centroid_coordinates ||
        (Nb > 0 && (!mesh->boundary_cells || !mesh->boundary_edges || !mesh->boundary_tag)))
        return fail(nullptr, SWGPU_EINVAL, "null mesh array");

    // ---- scenarios of an ensemble: 256-aligned ranges with no neighbour
    // across a range boundary
    std::vector<int> tri_scen;
    if (offsets) {
        if (nscen < 1 || offsets[0] != 0 || offsets[nscen] != N)
            return fail(nullptr, SWGPU_EINVAL,
                        "scenario offsets must start at 0 and end at the triangle count");
        tri_scen.resize((size_t)N);
        for (int s = 0; s < nscen; s++) {
            if (offsets[s + 1] <= offsets[s] || offsets[s] % 256 != 0 || offsets[s + 1] % 256 != 0)
                return fail(nullptr, SWGPU_EINVAL,
                            "scenario %d: range [%lld, %lld) must be non-empty and 256-aligned",
                            s, (long long)offsets[s], (long long)offsets[s + 1]);
            for (int64_t k = offsets[s]; k < offsets[s + 1]; k++) tri_scen[(size_t)k] = s;
        }
        for (int64_t k = 0; k < N; k++)
            for (int i = 0; i < 3; i++) {
                const int64_t n = mesh->neighbours[3 * k + i];
                const int64_t sn = mesh->surrogate_neighbours[3 * k + i];
                if ((n >= 0 && n < N && tri_scen[(size_t)n] != tri_scen[(size_t)k]) ||
                    (sn >= 0 && sn < N && tri_scen[(size_t)sn] != tri_scen[(size_t)k]))
                    return fail(nullptr, SWGPU_EMESH,
                                "triangle %lld has a neighbour in another scenario",
                                (long long)k);
            }
    }

    // ---- validate and pack the topology on the host
    std::vector<int> nbr((size_t)3 * N), surr((size_t)3 * N);
    std::vector<uint8_t> nb((size_t)N), order((size_t)N), full((size_t)N);
    int64_t maxtag = -1;
    for (int64_t m = 0; m < Nb; m++) {
        const int64_t c = mesh->boundary_cells[m], e = mesh->boundary_edges[m],
                      t = mesh->boundary_tag[m];
        if (c < 0 || c >= N || e < 0 || e > 2 || t < 0 || t > 1000000)
            return fail(nullptr, SWGPU_EMESH, "boundary slot %lld out of range", (long long)m);
        if (mesh->neighbours[3 * c + e] != -m - 1)
            return fail(nullptr, SWGPU_EMESH,
                        "boundary slot %lld: neighbours[%lld,%lld] is not -%lld-1", (long long)m,
                        (long long)c, (long long)e, (long long)m);
        maxtag = std::max(maxtag, t);
    }
    for (int64_t k = 0; k < N; k++) {
        int nbc = 0;
        for (int i = 0; i < 3; i++) {
            const int64_t n = mesh->neighbours[3 * k + i];
            const int64_t s = mesh->surrogate_neighbours[3 * k + i];
            if (s < 0 || s >= N)
                return fail(nullptr, SWGPU_EMESH, "surrogate neighbour of %lld out of range",
                            (long long)k);
            surr[(size_t)i * N + k] = (int)s;
            if (n >= 0) {
                const int64_t m = mesh->neighbour_edges[3 * k + i];
                if (n >= N || m < 0 || m > 2 || mesh->neighbours[3 * n + m] != k)
                    return fail(nullptr, SWGPU_EMESH,
                                "neighbour %lld of triangle %lld edge %d is inconsistent",
                                (long long)n, (long long)k, i);
                nbr[(size_t)i * N + k] = pack_neighbour((int)n, (int)m);
            } else {
                if (-n - 1 >= Nb)
                    return fail(nullptr, SWGPU_EMESH, "boundary index of %lld out of range",
                                (long long)k);
                nbr[(size_t)i * N + k] = (int)n;
                nbc++;
            }
        }
        if (mesh->number_of_boundaries[k] != nbc)
            return fail(nullptr, SWGPU_EMESH, "number_of_boundaries[%lld] != %d", (long long)k,
                        nbc);
        nb[k] = (uint8_t)nbc;
        full[k] = mesh->tri_full_flag ? (mesh->tri_full_flag[k] == 1) : 1;
        // ANUGA's summation order for triangle k: edges to lower-index
        // neighbours by neighbour index, then the other edges by index
        int idx[3] = {0, 1, 2}, cnt = 0, perm[3];
        for (int i = 0; i < 3; i++) {
            const int64_t n = mesh->neighbours[3 * k + i];
            if (n >= 0 && n < k) perm[cnt++] = i;
        }
        std::sort(perm, perm + cnt, [&](int a, int b) {
            return mesh->neighbours[3 * k + a] < mesh->neighbours[3 * k + b];
        });
        for (int i = 0; i < 3; i++) {
            const int64_t n = mesh->neighbours[3 * k + i];
            if (!(n >= 0 && n < k)) perm[cnt++] = idx[i];
        }
        order[k] = (uint8_t)(perm[0] | (perm[1] << 2) | (perm[2] << 4));
    }

    h = new Handle();
    h->precision = precision;
    int rc;
    {
        cudaError_t e = cudaGetDevice(&h->device);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            fail(nullptr, SWGPU_ECUDA, "no CUDA device: %s", cudaGetErrorString(e));
            delete h;
            return SWGPU_ECUDA;
        }
    }
#define TRY(x)                                      \
    do {                                            \
        rc = (x);                                   \
        if (rc) {                                   \
            g_create_error = h->err;                \
            swgpu_destroy(h);                       \
            return rc;                              \
        }                                           \
    } while (0)

    const size_t n1 = N, n3 = 3 * N, n6 = 6 * N, nb1 = Nb;
    DevMesh &M = h->M;
    M.N = (int)N;
    M.n_launch = (int)N;
    M.Nb = (int)Nb;
    int *d_nbr, *d_surr, *d_bcell, *d_bedge, *d_btag;
    uint8_t *d_nb, *d_order, *d_full;
    double *d_normals, *d_len, *d_radii, *d_areas, *d_vxy, *d_cxy;
    TRY(dalloc(h, &d_nbr, n3));
    TRY(dalloc(h, &d_surr, n3));
    TRY(dalloc(h, &d_nb, n1));
    TRY(dalloc(h, &d_order, n1));
    TRY(dalloc(h, &d_full, n1));
    TRY(dalloc(h, &d_normals, n6));
    TRY(dalloc(h, &d_len, n3));
    TRY(dalloc(h, &d_radii, n1));
    TRY(dalloc(h, &d_areas, n1));
    TRY(dalloc(h, &d_vxy, n6));
    TRY(dalloc(h, &d_cxy, 2 * n1));
    TRY(dalloc(h, &d_bcell, nb1));
    TRY(dalloc(h, &d_bedge, nb1));
    TRY(dalloc(h, &d_btag, nb1));
    TRY(upload(h, d_nbr, nbr.data(), n3));
    TRY(upload(h, d_surr, surr.data(), n3));
    TRY(upload(h, d_nb, nb.data(), n1));
    TRY(upload(h, d_order, order.data(), n1));
    TRY(upload(h, d_full, full.data(), n1));
    h->h_normals = to_planes<double>(mesh->normals, N, 6);
    h->h_len = to_planes<double>(mesh->edgelengths, N, 3);
    h->h_vxy = to_planes<double>(mesh->vertex_coordinates, N, 6);
    h->h_cxy = to_planes<double>(mesh->centroid_coordinates, N, 2);
    h->h_areas.assign(mesh->areas, mesh->areas + N);
    h->h_radii.assign(mesh->radii, mesh->radii + N);
    h->h_nbr = nbr;
    h->h_surr = surr;
    h->h_nb = nb;
    TRY(upload(h, d_normals, h->h_normals.data(), n6));
    TRY(upload(h, d_len, h->h_len.data(), n3));
    TRY(upload(h, d_radii, mesh->radii, n1));
    TRY(upload(h, d_areas, mesh->areas, n1));
    TRY(upload(h, d_vxy, h->h_vxy.data(), n6));
    TRY(upload(h, d_cxy, h->h_cxy.data(), 2 * n1));
    if (Nb > 0) {
        std::vector<int> bc(Nb), be(Nb), bt(Nb);
        for (int64_t m = 0; m < Nb; m++) {
            bc[m] = (int)mesh->boundary_cells[m];
            be[m] = (int)mesh->boundary_edges[m];
            bt[m] = (int)mesh->boundary_tag[m];
        }
        TRY(upload(h, d_bcell, bc.data(), nb1));
        TRY(upload(h, d_bedge, be.data(), nb1));
        TRY(upload(h, d_btag, bt.data(), nb1));
    }
    M.nbr = d_nbr;
    M.surr = d_surr;
    M.nb = d_nb;
    M.order = d_order;
    M.full = d_full;
    M.normals = d_normals;
    M.len = d_len;
    M.radii = d_radii;
    M.areas = d_areas;
    M.vxy = d_vxy;
    M.cxy = d_cxy;
    M.bcell = d_bcell;
    M.bedge = d_bedge;
    M.btag = d_btag;

    // ---- quantities
    DevState &S = h->S;
    TRY(dalloc(h, &S.w, n1));
    TRY(dalloc(h, &S.uh, n1));
    TRY(dalloc(h, &S.vh, n1));
    TRY(dalloc(h, &S.zc, n1));
    TRY(dalloc(h, &S.fric, n1));
    TRY(dalloc(h, &S.uvel, n1));
    TRY(dalloc(h, &S.vvel, n1));
    TRY(dalloc(h, &S.zv, n3));
    TRY(dalloc(h, &S.ze, n3));
    TRY(dalloc(h, &S.wb, nb1));
    TRY(dalloc(h, &S.uhb, nb1));
    TRY(dalloc(h, &S.vhb, nb1));
    TRY(dalloc(h, &S.zb, nb1));
    TRY(dalloc(h, &S.hc, n1));
    TRY(dalloc(h, &S.uc, n1));
    TRY(dalloc(h, &S.vc, n1));
    TRY(dalloc(h, &S.hb, nb1));
    TRY(dalloc(h, &S.ub, nb1));
    TRY(dalloc(h, &S.vb, nb1));
    TRY(dalloc(h, &S.partials, (size_t)grid_for((int)N) + 1));
    TRY(dalloc(h, &S.bw, n1));   // Runge-Kutta backups
    TRY(dalloc(h, &S.buh, n1));
    TRY(dalloc(h, &S.bvh, n1));
    TRY(dalloc(h, &S.we, n3));
    TRY(dalloc(h, &S.uhe, n3));
    TRY(dalloc(h, &S.vhe, n3));
    if (precision == SWGPU_FP64) {
        TRY(dalloc(h, &S.wv, n3));
        TRY(dalloc(h, &S.uhv, n3));
        TRY(dalloc(h, &S.vhv, n3));
        TRY(dalloc(h, &S.ew, n1));
        TRY(dalloc(h, &S.euh, n1));
        TRY(dalloc(h, &S.evh, n1));
        TRY(dalloc(h, &S.suh, n1));
        TRY(dalloc(h, &S.svh, n1));
        TRY(dalloc(h, &S.max_speed, n1));
    } else {
        DevMixed &X = h->X;
        X.S = (int)(((size_t)N + 63) / 64 * 64);
        const size_t s1 = X.S, s3 = 3 * s1;
        TRY(dalloc(h, &X.hd, s1));
        TRY(dalloc(h, &X.ws, s1));
        TRY(dalloc(h, &X.hf, s1));
        TRY(dalloc(h, &X.vel, s1));
        TRY(dalloc(h, &X.es, s3));
        TRY(dalloc(h, &X.hbf, nb1));
        TRY(dalloc(h, &X.uhbf, nb1));
        TRY(dalloc(h, &X.vhbf, nb1));
        TRY(dalloc(h, &X.wjb, nb1));
        TRY(dalloc(h, &X.ewu, s1));
        TRY(dalloc(h, &X.evh, s1));
        TRY(dalloc(h, &X.nrm, s3));
        TRY(dalloc(h, &X.lnb, s3));
        TRY(dalloc(h, &X.rad, s1));
        TRY(dalloc(h, &X.gc, s3));
        TRY(dalloc(h, &X.dzv, s3));
        TRY(dalloc(h, &X.dze, s3));
        TRY(dalloc(h, &X.ust, s1));
        TRY(dalloc(h, &X.kind, s1));
        TRY(dalloc(h, &X.surrp, s3));
        CK(cudaMemcpy2DAsync(X.surrp, X.S * sizeof(int), M.surr, (size_t)N * sizeof(int),
                             (size_t)N * sizeof(int), 3, cudaMemcpyDeviceToDevice, h->stream));
        // FP64 vertex planes are kept for downloads (stage = depth + bed)
        TRY(dalloc(h, &S.wv, n3));
        TRY(dalloc(h, &S.uhv, n3));
        TRY(dalloc(h, &S.vhv, n3));
    }

    // ---- parameters, boundary tags, control block
    DevParams &P = h->P;
    P.g = params->g;
    P.epsilon = params->epsilon;
    P.H0 = params->H0;
    P.minimum_allowed_height = params->minimum_allowed_height;
    P.maximum_allowed_speed = params->maximum_allowed_speed;
    P.beta_w = params->beta_w;
    P.beta_w_dry = params->beta_w_dry;
    P.beta_uh = params->beta_uh;
    P.beta_uh_dry = params->beta_uh_dry;
    P.beta_vh = params->beta_vh;
    P.beta_vh_dry = params->beta_vh_dry;
    P.alpha_balance = params->alpha_balance;
    P.CFL = params->CFL;
    P.evolve_max_timestep = params->evolve_max_timestep;
    P.evolve_min_timestep = params->evolve_min_timestep;
    P.tight_slope_limiters = (int)params->tight_slope_limiters;
    P.use_centroid_velocities = (int)params->use_centroid_velocities;
    P.optimise_dry_cells = (int)params->optimise_dry_cells;
    P.extrapolate_velocity_second_order = (int)params->extrapolate_velocity_second_order;
    P.use_sloped_mannings = (int)params->use_sloped_mannings;
    P.max_smallsteps = (int)params->max_smallsteps;
    P.default_order = (int)params->default_order;
    P.flow_algorithm = params->flow_algorithm ? 1 : 0;
    P.limiter = params->use_edge_limiter ? kLimiterEdge
                : params->optimised_gradient_limiter ? kLimiterOptimised
                                                     : kLimiterVertex;
    P.f_g = (float)P.g;
    P.f_eps = (float)P.epsilon;
    P.f_H0 = (float)P.H0;
    P.f_h0 = (float)(P.H0 * P.H0);
    P.f_lim = (float)(10 * P.H0);
    P.f_mah = (float)P.minimum_allowed_height;
    P.f_mas = (float)P.maximum_allowed_speed;
    P.f_max_dt = (float)std::min(P.evolve_max_timestep, 3.0e38);
    P.f_alpha = (float)P.alpha_balance;
    P.f_beta_w = (float)P.beta_w;
    P.f_beta_w_dry = (float)P.beta_w_dry;
    P.f_beta_uh = (float)P.beta_uh;
    P.f_beta_uh_dry = (float)P.beta_uh_dry;
    P.f_beta_vh = (float)P.beta_vh;
    P.f_beta_vh_dry = (float)P.beta_vh_dry;
    if (!(P.evolve_max_timestep > 0) || (P.default_order != 1 && P.default_order != 2)) {
        fail(h, SWGPU_EINVAL, "evolve_max_timestep must be > 0 and default_order 1 or 2");
        g_create_error = h->err;
        swgpu_destroy(h);
        return SWGPU_EINVAL;
    }
    if (P.flow_algorithm != 0 && precision != SWGPU_FP64) {
        fail(h, SWGPU_EINVAL, "the 'tsunami' flow algorithm runs in FP64 precision only");
        g_create_error = h->err;
        swgpu_destroy(h);
        return SWGPU_EINVAL;
    }
    if (P.limiter != kLimiterOptimised && precision != SWGPU_FP64) {
        fail(h, SWGPU_EINVAL,
             "the per-quantity vertex / edge limiters (optimised_gradient_limiter = 0 or "
             "use_edge_limiter = 1) run in FP64 precision only");
        g_create_error = h->err;
        swgpu_destroy(h);
        return SWGPU_EINVAL;
    }

    h->ntags = (int)(maxtag + 1);
    h->nscen = offsets ? nscen : 1;
    TRY(dalloc(h, &h->d_tags, (size_t)std::max(h->ntags, 1)));  // zero = reflective
    TRY(dalloc(h, &h->d_ctrl, (size_t)h->nscen));
    TRY(dalloc(h, &h->d_summary, 1));
    const int nwords = (h->nscen + 31) / 32;
    TRY(dalloc(h, &h->d_halt_bits, (size_t)nwords));
    TRY(dalloc(h, &h->d_scalar, 4));
    if (offsets) {
        const int64_t nblk = N / 256;
        std::vector<int> blk((size_t)nblk);
        for (int64_t b = 0; b < nblk; b++) blk[(size_t)b] = tri_scen[(size_t)(b * 256)];
        TRY(dalloc(h, &h->d_blk_scen, (size_t)nblk));
        TRY(upload(h, h->d_blk_scen, blk.data(), (size_t)nblk));
        M.blk_scen = h->d_blk_scen;
        h->scen_offsets.assign(offsets, offsets + nscen + 1);
    }
    {
        cudaError_t e = cudaMallocHost((void **)&h->h_ctrl, sizeof(Ctrl) * h->nscen);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&h->h_summary, sizeof(RunSummary));
        if (e == cudaSuccess)
            e = cudaMallocHost((void **)&h->h_halt_bits, sizeof(unsigned) * ((h->nscen + 31) / 32));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&h->h_scalar, 4 * sizeof(double));
        if (e != cudaSuccess) {
            fail(h, SWGPU_ENOMEM, "pinned host allocation: %s", cudaGetErrorString(e));
            g_create_error = h->err;
            swgpu_destroy(h);
            return SWGPU_ENOMEM;
        }
    }
    std::memset(h->h_ctrl, 0, sizeof(Ctrl) * h->nscen);
    std::memset(h->h_summary, 0, sizeof(RunSummary));
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
        // the mixed flux's tile: 256 triangles on meshes of many waves (fewer,
        // longer blocks: 0.9% faster at 4M), 128 on small ones (more blocks
        // for the latency-bound case: 3% faster at 40k)
        const int flux_tile = N >= (int64_t(1) << 20) ? 256 : 128;
        M.shape = LaunchShape{precision == SWGPU_MIXED ? flux_tile : kBlock, kBlock, kBlock, 0,
                              std::max(sms, 1), 1};
    }
    for (int i = 0; i < h->nscen; i++) {
        Ctrl *c = &h->h_ctrl[i];
        c->order = P.default_order;
        c->finaltime = -1.0;
        c->yieldtime = 1.0e300;
        c->yieldstep = 1.0e300;
        c->time_epsilon = params->epsilon;
        c->rec_max = P.evolve_min_timestep;
        c->rec_min = P.evolve_max_timestep;
        c->budget = -1;
        c->summary = h->d_summary;
        c->halt_bits = h->d_halt_bits;
        c->scen = i;
        reset_ftmin(c, P);
    }
    set_block_counts(h);
    TRY(push_ctrl(h));
    TRY(upload(h, h->d_summary, h->h_summary, 1));
    if (precision == SWGPU_MIXED) TRY(build_mixed_geometry(h) ? fail(h, SWGPU_ECUDA, "mixed geometry upload") : SWGPU_OK);
    *handle_out = h;
#undef TRY
    return SWGPU_OK;
}

int swgpu_create(const swgpu_mesh *mesh, const swgpu_params *params, int precision,
                 void **handle_out) {
    return create_impl(mesh, params, precision, nullptr, 1, handle_out);
}

int swgpu_create_ensemble(const swgpu_mesh *mesh, const int64_t *scenario_offsets, int nscen,
                          const swgpu_params *params, int precision, void **handle_out) {
    if (!scenario_offsets || nscen < 1)
        return fail(nullptr, SWGPU_EINVAL, "an ensemble needs scenario offsets");
    return create_impl(mesh, params, precision, scenario_offsets, nscen, handle_out);
}

int swgpu_destroy(void *handle) {
    if (!handle) return SWGPU_OK;
    Handle *h = static_cast<Handle *>(handle);
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    for (void *p : h->allocs) cudaFree(p);
    if (h->h_ctrl) cudaFreeHost(h->h_ctrl);
    if (h->h_summary) cudaFreeHost(h->h_summary);
    if (h->h_halt_bits) cudaFreeHost(h->h_halt_bits);
    if (h->h_scalar) cudaFreeHost(h->h_scalar);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SWGPU_OK;
}

int swgpu_set_boundary_tags(void *handle, const swgpu_boundary_tag *tags, int ntags) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || (!tags && ntags > 0)) return fail(h, SWGPU_EINVAL, "null argument");
    if (ntags < h->ntags)
        return fail(h, SWGPU_EINVAL, "mesh uses %d boundary tags, %d given", h->ntags, ntags);
    std::vector<BcTag> t((size_t)ntags);
    for (int i = 0; i < ntags; i++) {
        if (tags[i].type < SWGPU_BC_REFLECTIVE || tags[i].type > SWGPU_BC_TIME_STAGE_FOURIER)
            return fail(h, SWGPU_EBOUNDARY, "tag %d: unknown boundary type %lld", i,
                        (long long)tags[i].type);
        if (tags[i].type == SWGPU_BC_TIME_STAGE_SINE && !(tags[i].p[2] != 0.0))
            return fail(h, SWGPU_EINVAL, "tag %d: sine boundary needs a nonzero period", i);
        if (tags[i].type == SWGPU_BC_TIME_STAGE_FOURIER && !(tags[i].p[5] != 0.0))
            return fail(h, SWGPU_EINVAL, "tag %d: Fourier boundary needs a nonzero period", i);
        if (tags[i].type == SWGPU_BC_INFLOW_HYDROGRAPH &&
            !(tags[i].p[0] >= 0.0 && tags[i].p[1] > 0.0 && tags[i].p[2] > 0.0))
            return fail(h, SWGPU_EINVAL,
                        "tag %d: hydrograph needs peak >= 0 and positive rise and fall", i);
        t[i].type = (int)tags[i].type;
        for (int j = 0; j < 8; j++) t[i].p[j] = tags[i].p[j];
    }
    const int n = std::max(h->ntags, 1);
    return upload(h, h->d_tags, t.data(), (size_t)std::min(ntags, n));
}

int swgpu_set_quantity(void *handle, int q, const double *centroid, const double *vertex,
                       const double *edge) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !centroid) return fail(h, SWGPU_EINVAL, "null argument");
    const int64_t N = h->M.N;
    DevState &S = h->S;
    double *c = nullptr, *v = nullptr, *e = nullptr;
    switch (q) {
        case SWGPU_STAGE: c = S.w; v = S.wv; e = S.we; break;
        case SWGPU_XMOMENTUM: c = S.uh; v = S.uhv; e = S.uhe; break;
        case SWGPU_YMOMENTUM: c = S.vh; v = S.vhv; e = S.vhe; break;
        case SWGPU_ELEVATION: c = S.zc; v = S.zv; e = S.ze; break;
        case SWGPU_FRICTION: c = S.fric; break;
        default: return fail(h, SWGPU_EINVAL, "quantity %d cannot be set", q);
    }
    int rc = upload(h, c, centroid, (size_t)N);
    if (rc) return rc;
    if (v && vertex) {
        auto pv = to_planes<double>(vertex, N, 3);
        if ((rc = upload(h, v, pv.data(), (size_t)3 * N))) return rc;
    }
    if (e && edge) {
        auto pe = to_planes<double>(edge, N, 3);
        if ((rc = upload(h, e, pe.data(), (size_t)3 * N))) return rc;
    } else if (q == SWGPU_ELEVATION && vertex) {
        // quantity.c:687-706: bed edge values from the bed vertex values
        std::vector<double> pe((size_t)3 * N);
        for (int64_t k = 0; k < N; k++) {
            const double q0 = vertex[3 * k], q1 = vertex[3 * k + 1], q2 = vertex[3 * k + 2];
            pe[k] = 0.5 * (q1 + q2);
            pe[N + k] = 0.5 * (q0 + q2);
            pe[2 * N + k] = 0.5 * (q0 + q1);
        }
        if ((rc = upload(h, e, pe.data(), (size_t)3 * N))) return rc;
    }
    if (q == SWGPU_ELEVATION) h->elevation_set = true;
    if (h->precision == SWGPU_MIXED && (q == SWGPU_ELEVATION || q == SWGPU_FRICTION)) {
        if (build_mixed_geometry(h)) return fail(h, SWGPU_ECUDA, "mixed geometry upload");
    }
    if (q == SWGPU_STAGE || q == SWGPU_ELEVATION) h->mixed_from_stage = true;
    if (q <= SWGPU_YMOMENTUM) h->vertices_stale = true;
    return SWGPU_OK;
}

int swgpu_get_quantity(void *handle, int q, double *centroid, double *vertex, double *edge) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    const int64_t N = h->M.N;
    DevState &S = h->S;
    int rc;
    if (h->precision == SWGPU_MIXED && !h->mixed_from_stage) {
        // the FP64 views of the mixed state: vertex and edge values when
        // asked for, else the centroid stage alone (momentum is FP64 state)
        if ((vertex || edge) && q <= SWGPU_YMOMENTUM) {
            launch_vertices_from_mixed(h->M, h->S, h->X, h->stream);
            if ((rc = check_launch(h, "mixed vertex values"))) return rc;
        } else if (q == SWGPU_STAGE || q >= SWGPU_HEIGHT) {
            launch_stage_from_mixed(h->M, h->S, h->X, h->stream);
            if ((rc = check_launch(h, "mixed centroid stage"))) return rc;
        }
    }
    // the 'tsunami' distribute stores its extrapolated edge values, which are
    // not the interpolation of the vertex values
    if ((vertex || edge) && q <= SWGPU_YMOMENTUM && !h->P.flow_algorithm) {
        launch_interpolate_fp64(h->M, h->S, h->stream);
        if ((rc = check_launch(h, "interpolate"))) return rc;
    }
    const double *c = nullptr, *v = nullptr, *e = nullptr;
    switch (q) {
        case SWGPU_STAGE: c = S.w; v = S.wv; e = S.we; break;
        case SWGPU_XMOMENTUM: c = S.uh; v = S.uhv; e = S.uhe; break;
        case SWGPU_YMOMENTUM: c = S.vh; v = S.vhv; e = S.vhe; break;
        case SWGPU_ELEVATION: c = S.zc; v = S.zv; e = S.ze; break;
        case SWGPU_FRICTION: c = S.fric; break;
        case SWGPU_HEIGHT: c = S.hc; break;
        case SWGPU_XVELOCITY: c = S.uc; break;
        case SWGPU_YVELOCITY: c = S.vc; break;
        default: return fail(h, SWGPU_EINVAL, "unknown quantity %d", q);
    }
    if (q >= SWGPU_HEIGHT) {
        launch_other_quantities(h->M, h->S, h->stream);
        if ((rc = check_launch(h, "other quantities"))) return rc;
    }
    if (centroid && (rc = download(h, centroid, c, (size_t)N))) return rc;
    std::vector<double> tmp;
    auto planes_out = [&](double *dst, const double *src) -> int {
        tmp.resize((size_t)3 * N);
        int r = download(h, tmp.data(), src, (size_t)3 * N);
        if (r) return r;
        for (int64_t k = 0; k < N; k++)
            for (int i = 0; i < 3; i++) dst[3 * k + i] = tmp[(size_t)i * N + k];
        return SWGPU_OK;
    };
    if (vertex) {
        if (v) {
            if ((rc = planes_out(vertex, v))) return rc;
        } else if (centroid) {
            for (int64_t k = 0; k < N; k++)
                vertex[3 * k] = vertex[3 * k + 1] = vertex[3 * k + 2] = centroid[k];
        }
    }
    if (edge) {
        if (e) {
            if ((rc = planes_out(edge, e))) return rc;
        } else if (centroid) {
            for (int64_t k = 0; k < N; k++)
                edge[3 * k] = edge[3 * k + 1] = edge[3 * k + 2] = centroid[k];
        }
    }
    return SWGPU_OK;
}

int swgpu_get_boundary_values(void *handle, int q, double *out) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !out) return fail(h, SWGPU_EINVAL, "null argument");
    const double *src = nullptr;
    switch (q) {
        case SWGPU_STAGE: src = h->S.wb; break;
        case SWGPU_XMOMENTUM: src = h->S.uhb; break;
        case SWGPU_YMOMENTUM: src = h->S.vhb; break;
        case SWGPU_ELEVATION: src = h->S.zb; break;
        // derived: as of the last update_other_quantities
        case SWGPU_HEIGHT: src = h->S.hb; break;
        case SWGPU_XVELOCITY: src = h->S.ub; break;
        case SWGPU_YVELOCITY: src = h->S.vb; break;
        default: return fail(h, SWGPU_EINVAL, "no boundary values for quantity %d", q);
    }
    return download(h, out, src, (size_t)h->M.Nb);
}

static int require_fp64(Handle *h, const char *what) {
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (h->precision != SWGPU_FP64)
        return fail(h, SWGPU_EINVAL,
                    "%s is a per-method entry point of the FP64 path; mixed-precision "
                    "handles run whole steps only",
                    what);
    return SWGPU_OK;
}

int swgpu_get_explicit_update(void *handle, int q, double *out) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "explicit_update");
    if (rc) return rc;
    const double *src = q == SWGPU_STAGE ? h->S.ew : q == SWGPU_XMOMENTUM ? h->S.euh
                                                 : q == SWGPU_YMOMENTUM ? h->S.evh : nullptr;
    if (!src || !out) return fail(h, SWGPU_EINVAL, "bad quantity or null output");
    return download(h, out, src, (size_t)h->M.N);
}

int swgpu_get_max_speed(void *handle, double *out) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "max_speed");
    if (rc) return rc;
    if (!out) return fail(h, SWGPU_EINVAL, "null output");
    return download(h, out, h->S.max_speed, (size_t)h->M.N);
}

int swgpu_get_semi_implicit_update(void *handle, int q, double *out) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "semi_implicit_update");
    if (rc) return rc;
    if (!out) return fail(h, SWGPU_EINVAL, "null output");
    if (q == SWGPU_STAGE) {
        std::fill(out, out + h->M.N, 0.0);
        return SWGPU_OK;
    }
    const double *src = q == SWGPU_XMOMENTUM ? h->S.suh : q == SWGPU_YMOMENTUM ? h->S.svh : nullptr;
    if (!src) return fail(h, SWGPU_EINVAL, "bad quantity");
    return download(h, out, src, (size_t)h->M.N);
}

int swgpu_protect(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "protect");
    if (rc) return rc;
    launch_prepare_fp64(h->M, h->S, h->P, h->d_ctrl, h->stream);
    if ((rc = check_launch(h, "protect"))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_distribute_to_vertices_and_edges(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    int rc = sync_ctrl(h);  // current _order_ lives in the control block
    if (rc) return rc;
    if ((rc = issue_distribute(h, false))) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    return device_status(h);
}

int swgpu_update_boundary(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (h->precision == SWGPU_MIXED && !h->mixed_from_stage) {
        launch_vertices_from_mixed(h->M, h->S, h->X, h->stream);
    }
    launch_boundary_fp64(h->M, h->S, h->P, h->d_tags, h->d_ctrl, h->stream);
    int rc = check_launch(h, "update_boundary");
    if (rc) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    return device_status(h);
}

int swgpu_compute_fluxes(void *handle, double *flux_timestep) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "compute_fluxes");
    if (rc) return rc;
    if ((rc = require_single(h, "compute_fluxes"))) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    reset_ftmin(h->h_ctrl, h->P);
    if ((rc = push_ctrl(h))) return rc;
    launch_flux_fp64(h->M, h->S, h->P, h->d_ctrl, kWriteMaxSpeed, h->stream);
    if ((rc = check_launch(h, "compute_fluxes"))) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    double ft;
    std::memcpy(&ft, &h->h_ctrl->ftmin_bits, sizeof ft);
    h->h_ctrl->flux_timestep = ft;
    if ((rc = push_ctrl(h))) return rc;
    if (flux_timestep) *flux_timestep = ft;
    return device_status(h);
}

int swgpu_compute_forcing_terms(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "compute_forcing_terms");
    if (rc) return rc;
    launch_forcing_fp64(h->M, h->S, h->P, false, h->stream);
    if ((rc = check_launch(h, "compute_forcing_terms"))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_manning_friction_explicit(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "manning_friction_explicit");
    if (rc) return rc;
    launch_forcing_fp64(h->M, h->S, h->P, true, h->stream);
    if ((rc = check_launch(h, "manning_friction_explicit"))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_extrapolate_second_order_sw(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "extrapolate_second_order_sw");
    if (rc) return rc;
    if (h->P.flow_algorithm)
        return fail(h, SWGPU_EINVAL,
                    "extrapolate_second_order_sw: the 'tsunami' flow algorithm extrapolates "
                    "to edges inside distribute_to_vertices_and_edges");
    if (h->P.extrapolate_velocity_second_order) launch_velocities_fp64(h->M, h->S, h->P, h->stream);
    launch_distribute_fp64(h->M, h->S, h->P, h->d_tags, h->d_ctrl, kExtrapolateOnly, h->stream);
    if ((rc = check_launch(h, "extrapolate_second_order_sw"))) return rc;
    h->vertices_stale = false;
    if ((rc = sync_ctrl(h))) return rc;
    return device_status(h);
}

int swgpu_balance_deep_and_shallow(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "balance_deep_and_shallow");
    if (rc) return rc;
    launch_balance_fp64(h->M, h->S, h->P, h->stream);
    if ((rc = check_launch(h, "balance_deep_and_shallow"))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_update_conserved_quantities(void *handle, double timestep) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "update_conserved_quantities");
    if (rc) return rc;
    if ((rc = require_single(h, "update_conserved_quantities"))) return rc;
    launch_update_fp64(h->M, h->S, h->P, h->d_ctrl, timestep, 0, kEulerStage, h->stream);
    if ((rc = check_launch(h, "update_conserved_quantities"))) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    return device_status(h);
}

int swgpu_backup_conserved_quantities(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "backup_conserved_quantities");
    if (rc) return rc;
    const size_t bytes = sizeof(double) * (size_t)h->M.N;
    CK(cudaMemcpyAsync(h->S.bw, h->S.w, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->S.buh, h->S.uh, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->S.bvh, h->S.vh, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_saxpy_conserved_quantities(void *handle, double a, double b) {
    Handle *h = static_cast<Handle *>(handle);
    int rc = require_fp64(h, "saxpy_conserved_quantities");
    if (rc) return rc;
    launch_saxpy_fp64(h->M, h->S, a, b, h->stream);
    if ((rc = check_launch(h, "saxpy_conserved_quantities"))) return rc;
    h->vertices_stale = true;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_set_timestepping_method(void *handle, int method) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (method != SWGPU_EULER && method != SWGPU_RK2 && method != SWGPU_RK3)
        return fail(h, SWGPU_EINVAL, "timestepping method %d (1 euler, 2 rk2, 3 rk3)", method);
    if (method != h->timestepping_method) {
        CK(cudaStreamSynchronize(h->stream));
        drop_graphs(h);  // rebuilt with the new stages on the next run
    }
    h->timestepping_method = method;
    return SWGPU_OK;
}

int swgpu_update_other_quantities(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (h->precision == SWGPU_MIXED && !h->mixed_from_stage)
        launch_stage_from_mixed(h->M, h->S, h->X, h->stream);
    launch_other_quantities(h->M, h->S, h->stream);
    int rc = check_launch(h, "update_other_quantities");
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

int swgpu_mass(void *handle, double *mass) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !mass) return fail(h, SWGPU_EINVAL, "null argument");
    if (h->precision == SWGPU_MIXED && !h->mixed_from_stage)
        launch_mass_mixed(h->M, h->S, h->X, h->d_scalar, h->stream);
    else
        launch_mass(h->M, h->S, h->d_scalar, h->stream);
    int rc = check_launch(h, "mass");
    if (rc) return rc;
    return download(h, mass, h->d_scalar, 1);
}

int swgpu_get_state(void *handle, swgpu_state *state) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !state) return fail(h, SWGPU_EINVAL, "null argument");
    int rc = sync_ctrl(h);
    if (rc) return rc;
    fill_state(h->h_ctrl, state);
    return SWGPU_OK;
}

int swgpu_ensemble_get_state(void *handle, int scenario, swgpu_state *state) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !state) return fail(h, SWGPU_EINVAL, "null argument");
    if (scenario < 0 || scenario >= h->nscen)
        return fail(h, SWGPU_EINVAL, "scenario %d of %d", scenario, h->nscen);
    int rc = sync_ctrl(h);
    if (rc) return rc;
    fill_state(&h->h_ctrl[scenario], state);
    return SWGPU_OK;
}

int swgpu_ensemble_set_finaltimes(void *handle, const double *finaltimes) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !finaltimes) return fail(h, SWGPU_EINVAL, "null argument");
    int rc = sync_ctrl(h);
    if (rc) return rc;
    for (int i = 0; i < h->nscen; i++) {
        if (finaltimes[i] > 0 && finaltimes[i] < h->h_ctrl[i].time)
            return fail(h, SWGPU_EINVAL, "scenario %d: finaltime before its time", i);
        h->h_ctrl[i].finaltime = finaltimes[i] > 0 ? finaltimes[i] : -1.0;
    }
    return push_ctrl(h);
}

// Water volume of every scenario: the block partials of swgpu_mass summed
// per scenario in the order of the device's final reduction (strided
// per-thread sums over 256 threads, then a pairwise tree), so that each
// equals swgpu_mass of the scenario run alone.
int swgpu_ensemble_mass(void *handle, double *masses) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !masses) return fail(h, SWGPU_EINVAL, "null argument");
    if (h->precision == SWGPU_MIXED && !h->mixed_from_stage)
        launch_mass_partials_mixed(h->M, h->S, h->X, h->stream);
    else
        launch_mass_partials(h->M, h->S, h->stream);
    int rc = check_launch(h, "ensemble mass");
    if (rc) return rc;
    const int nblk = grid_for(h->M.N);
    std::vector<double> part((size_t)nblk);
    if ((rc = download(h, part.data(), h->S.partials, (size_t)nblk))) return rc;
    for (int i = 0; i < h->nscen; i++) {
        const int64_t b0 = h->nscen > 1 ? h->scen_offsets[i] / kBlock : 0;
        const int64_t nb = h->nscen > 1 ? h->scen_offsets[i + 1] / kBlock - b0 : nblk;
        double sh[kBlock];
        for (int t = 0; t < kBlock; t++) {
            double acc = 0.0;
            for (int64_t j = t; j < nb; j += kBlock) acc += part[(size_t)(b0 + j)];
            sh[t] = acc;
        }
        for (int w = kBlock / 2; w > 0; w >>= 1)
            for (int t = 0; t < w; t++) sh[t] += sh[t + w];
        masses[i] = sh[0];
    }
    return SWGPU_OK;
}

int swgpu_get_launch_config(void *handle, swgpu_launch_config *cfg) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !cfg) return fail(h, SWGPU_EINVAL, "null argument");
    cfg->flux_block = h->M.shape.flux;
    cfg->update_block = h->M.shape.update;
    cfg->distribute_block = h->M.shape.distribute;
    cfg->steps_per_graph = h->steps_per_graph;
    cfg->flux_pipelined = h->M.shape.pipelined;
    cfg->dependent_launch = h->M.shape.pdl;
    return SWGPU_OK;
}

int swgpu_set_launch_config(void *handle, const swgpu_launch_config *cfg) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !cfg) return fail(h, SWGPU_EINVAL, "null argument");
    auto one_of = [](int v, std::initializer_list<int> ok) {
        for (int x : ok)
            if (v == x) return true;
        return false;
    };
    // an ensemble scenario starts on a 256-triangle boundary: no block may
    // straddle two scenarios
    const int top = h->nscen > 1 ? 256 : 512;
    if (!one_of(cfg->flux_block, {64, 128, 256}) ||
        !one_of(cfg->update_block, {128, 256, 512}) ||
        !one_of(cfg->distribute_block, {128, 256, 512}) || cfg->update_block > top ||
        cfg->distribute_block > top || cfg->steps_per_graph < 1 || cfg->steps_per_graph > 64 ||
        (cfg->flux_pipelined && cfg->flux_block > 128))
        return fail(h, SWGPU_EINVAL,
                    "launch config: flux 64/128/256 (at most 128 pipelined), update and "
                    "distribute 128/256/512 (at most 256 for an ensemble), 1..64 steps per graph");
    int rc = sync_ctrl(h);
    if (rc) return rc;
    drop_graphs(h);  // recaptured with the new shape on the next run
    h->M.shape.flux = cfg->flux_block;
    h->M.shape.update = cfg->update_block;
    h->M.shape.distribute = cfg->distribute_block;
    h->M.shape.pipelined = cfg->flux_pipelined ? 1 : 0;
    h->M.shape.pdl = cfg->dependent_launch ? 1 : 0;
    h->steps_per_graph = cfg->steps_per_graph;
    set_block_counts(h);
    return push_ctrl(h);
}

int swgpu_set_tracking(void *handle, int on, double threshold) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (on && !(threshold >= 0.0)) return fail(h, SWGPU_EINVAL, "threshold must be >= 0");
    if (on) {
        if (!h->trk_hmax) {
            int rc = dalloc(h, &h->trk_hmax, (size_t)h->M.N);
            if (!rc) rc = dalloc(h, &h->trk_tarr, (size_t)h->M.N);
            if (rc) return rc;
        }
        h->S.hmax = h->trk_hmax;
        h->S.tarr = h->trk_tarr;
        h->P.track_threshold = threshold;
        launch_track_reset(h->M, h->S, h->stream);
        int rc = check_launch(h, "tracking reset");
        if (rc) return rc;
    } else {
        h->S.hmax = h->S.tarr = nullptr;  // the buffers stay for a later call
    }
    CK(cudaStreamSynchronize(h->stream));
    drop_graphs(h);  // recaptured with the new tracking state and threshold
    return SWGPU_OK;
}

int swgpu_get_tracking(void *handle, float *max_depth, float *arrival_time) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (!h->trk_hmax) return fail(h, SWGPU_EINVAL, "tracking was never switched on");
    int rc;
    if (max_depth && (rc = download(h, max_depth, h->trk_hmax, (size_t)h->M.N))) return rc;
    if (arrival_time && (rc = download(h, arrival_time, h->trk_tarr, (size_t)h->M.N))) return rc;
    return SWGPU_OK;
}

int swgpu_ensemble_size(void *handle, int *nscen) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !nscen) return fail(h, SWGPU_EINVAL, "null argument");
    *nscen = h->nscen;
    return SWGPU_OK;
}

int swgpu_set_state(void *handle, const swgpu_state *s) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !s) return fail(h, SWGPU_EINVAL, "null argument");
    if (s->order != 1 && s->order != 2) return fail(h, SWGPU_EINVAL, "order must be 1 or 2");
    int rc = sync_ctrl(h);
    if (rc) return rc;
    Ctrl *c = h->h_ctrl;
    c->time = s->time;
    c->yieldtime = s->yieldtime;
    c->finaltime = s->finaltime;
    c->timestep = s->timestep;
    c->flux_timestep = s->flux_timestep;
    c->rec_max = s->recorded_max_timestep;
    c->rec_min = s->recorded_min_timestep;
    c->order = s->order;
    c->smallsteps = s->smallsteps;
    c->steps_since_yield = s->number_of_steps;
    c->total_steps = s->total_steps;
    c->stop_reason = (int)s->stop_reason;
    c->status = (int)s->status;
    return push_ctrl(h);
}

int swgpu_evolve_start(void *handle, double starttime, double yieldstep, double finaltime) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    if (!(yieldstep > 0)) return fail(h, SWGPU_EINVAL, "yieldstep must be > 0");
    if (finaltime > 0 && finaltime < starttime)
        return fail(h, SWGPU_EINVAL, "finaltime before starttime");
    int rc = sync_ctrl(h);
    if (rc) return rc;
    // first distribute with the current order (gpu_domain_advanced.py:2476)
    if ((rc = issue_distribute(h, false))) return rc;
    if ((rc = sync_ctrl(h))) return rc;
    for (int i = 0; i < h->nscen; i++) {
        Ctrl *c = &h->h_ctrl[i];
        c->time = starttime;
        c->order = h->P.default_order;
        c->finaltime = finaltime > 0 ? finaltime : -1.0;
        c->yieldstep = yieldstep;
        c->yieldtime = starttime + yieldstep;
        c->rec_min = h->P.evolve_max_timestep;
        c->rec_max = h->P.evolve_min_timestep;
        c->steps_since_yield = 0;
        c->total_steps = 0;
        c->halt = 0;
        c->halt_pending = 0;
        c->stop_reason = kStopNone;
        c->status = 0;
        c->budget = -1;
        c->done_update = c->done_distribute = 0;
        reset_ftmin(c, h->P);
    }
    if ((rc = push_ctrl(h))) return rc;
    // update_ghosts (no-op), distribute, update_boundary (:2540-2543)
    if ((rc = issue_distribute(h, true))) return rc;
    h->resume_after_yield = false;
    if ((rc = sync_ctrl(h))) return rc;
    return device_status(h);
}

// Triangles the fused-step kernels are launched over; a change drops the
// captured graph (the stream must be idle).
static int set_launch_extent(Handle *h, int n) {
    if (h->M.n_launch == n) return SWGPU_OK;
    if (h->graph) {
        CK(cudaStreamSynchronize(h->stream));
        drop_graphs(h);
    }
    h->M.n_launch = n;
    return SWGPU_OK;
}

// Before a run: every scenario that has not reached its finaltime runs;
// those that stopped at a yield move to the next yield point
// (gpu_domain_advanced.py:2649-2654).
static int prepare_run(Handle *h, int64_t max_steps) {
    int rc = sync_ctrl(h);
    if (rc) return rc;
    if ((rc = device_status(h))) return rc;
    int running = 0;
    for (int i = 0; i < h->nscen; i++) {
        Ctrl *c = &h->h_ctrl[i];
        if (c->stop_reason == kStopFinal) {
            c->halt = 1;  // stays halted; counts as halted for the run
            continue;
        }
        if (h->resume_after_yield && c->stop_reason == kStopYield) {
            c->yieldtime += c->yieldstep;
            c->rec_min = h->P.evolve_max_timestep;
            c->rec_max = h->P.evolve_min_timestep;
            c->steps_since_yield = 0;
        }
        c->halt = 0;
        c->halt_pending = 0;
        c->stop_reason = kStopNone;
        c->budget = max_steps > 0 ? max_steps : -1;
        running++;
    }
    h->resume_after_yield = false;
    if (running == 0) return fail(h, SWGPU_EINVAL, "evolve already reached finaltime");
    h->h_summary->halted = h->nscen - running;
    h->h_summary->status = 0;
    if ((rc = upload(h, h->d_summary, h->h_summary, 1))) return rc;
    const int nwords = (h->nscen + 31) / 32;
    for (int w = 0; w < nwords; w++) h->h_halt_bits[w] = 0u;
    for (int i = 0; i < h->nscen; i++)
        if (h->h_ctrl[i].halt) h->h_halt_bits[i >> 5] |= 1u << (i & 31);
    if ((rc = upload(h, h->d_halt_bits, h->h_halt_bits, (size_t)nwords))) return rc;
    if ((rc = set_launch_extent(h, h->M.N))) return rc;
    return push_ctrl(h);
}

static int finish_run(Handle *h, swgpu_state *state) {
    int rc = sync_ctrl(h);
    if (rc) return rc;
    if ((rc = set_launch_extent(h, h->M.N))) return rc;
    for (int i = 0; i < h->nscen; i++)
        if (h->h_ctrl[i].stop_reason == kStopYield) h->resume_after_yield = true;
    if (state) fill_state(h->h_ctrl, state);
    return device_status(h);
}

static int run_graphs(Handle *h, int64_t max_steps, swgpu_state *state, double *elapsed_ms);

int swgpu_evolve_run(void *handle, int64_t max_steps, swgpu_state *state) {
    return run_graphs(static_cast<Handle *>(handle), max_steps, state, nullptr);
}

int swgpu_evolve_run_timed(void *handle, int64_t max_steps, swgpu_state *state,
                           double *elapsed_ms) {
    Handle *h = static_cast<Handle *>(handle);
    if (!elapsed_ms) return fail(h, SWGPU_EINVAL, "null elapsed_ms");
    return run_graphs(h, max_steps, state, elapsed_ms);
}

int swgpu_profile_steps(void *handle, int64_t nsteps, double *ms) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h || !ms || nsteps <= 0) return fail(h, SWGPU_EINVAL, "bad argument");
    int rc = prepare_run(h, nsteps);
    if (rc) return rc;
    // events around each kernel: flux, step clock (mixed), update, distribute
    cudaEvent_t ev[5];
    for (int i = 0; i < 5; i++) CK(cudaEventCreate(&ev[i]));
    double acc[4] = {0, 0, 0, 0};
    const bool mixed = h->precision != SWGPU_FP64;
    for (int64_t s = 0; s < nsteps; s++) {
        CK(cudaEventRecord(ev[0], h->stream));
        if (!mixed)
            launch_flux_fp64(h->M, h->S, h->P, h->d_ctrl, kFused, h->stream);
        else
            launch_flux_mixed(h->M, h->S, h->X, h->P, h->d_ctrl, kFused, h->stream);
        CK(cudaEventRecord(ev[1], h->stream));
        if (mixed) launch_step_clock_mixed(h->P, h->d_ctrl, h->nscen, h->M.shape.pdl, h->stream);
        CK(cudaEventRecord(ev[2], h->stream));
        if (!mixed)
            launch_update_fp64(h->M, h->S, h->P, h->d_ctrl, 0.0, kFused | kFrictionInline,
                               kEulerStage, h->stream);
        else
            launch_update_mixed(h->M, h->S, h->X, h->P, h->d_ctrl, kFused | kFrictionInline,
                                kEulerStage, h->stream);
        CK(cudaEventRecord(ev[3], h->stream));
        if (!mixed)
            launch_distribute_fp64(h->M, h->S, h->P, h->d_tags, h->d_ctrl,
                                   kFused | kWriteBoundary, h->stream);
        else
            launch_distribute_mixed(h->M, h->S, h->X, h->P, h->d_tags, h->d_ctrl,
                                    kFused | kWriteBoundary, kEulerStage, h->stream);
        CK(cudaEventRecord(ev[4], h->stream));
        if ((rc = check_launch(h, "profile step"))) return rc;
        CK(cudaEventSynchronize(ev[4]));
        float t;
        for (int i = 0; i < 4; i++) {
            CK(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
            acc[i] += t;
        }
    }
    for (int i = 0; i < 5; i++) cudaEventDestroy(ev[i]);
    // ms[0] flux, ms[1] update, ms[2] distribute, ms[3] step clock
    ms[0] = acc[0];
    ms[1] = acc[2];
    ms[2] = acc[3];
    ms[3] = acc[1];
    return finish_run(h, nullptr);
}

static int run_graphs(Handle *h, int64_t max_steps, swgpu_state *state, double *elapsed_ms) {
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    int rc = prepare_run(h, max_steps);
    if (rc) return rc;
    if ((rc = build_graph(h))) return rc;
    // with a step budget the device stops itself after max_steps steps; the
    // host issues max_steps / steps-per-graph whole graphs and then the
    // remaining steps' kernels one by one (no capture for a remainder that
    // may differ between runs), so that no step is issued beyond the budget
    const int spg = h->steps_per_graph;
    const int64_t full_graphs = max_steps > 0 ? max_steps / spg : INT64_MAX;
    const int tail = max_steps > 0 ? (int)(max_steps % spg) : 0;
    const int64_t max_graphs = max_steps > 0 ? full_graphs + (tail ? 1 : 0) : INT64_MAX;
    // keep two graphs in flight: while graph i runs, the host waits on the
    // control-block copy that follows graph i-1
    cudaEvent_t ev[2], t0, t1;
    CK(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
    CK(cudaEventCreate(&t0));
    CK(cudaEventCreate(&t1));
    CK(cudaEventRecord(t0, h->stream));
    int64_t launched = 0;
    cudaError_t e = cudaSuccess;
    int inflight = 0, slot = 0;
    bool halted = false;
    while (!halted && launched < max_graphs) {
        if (launched < full_graphs) {
            e = cudaGraphLaunch(h->graph, h->stream);
        } else {
            for (int s = 0; s < tail; s++) issue_step(h);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) break;
        e = cudaMemcpyAsync(h->h_summary, h->d_summary, sizeof(RunSummary),
                            cudaMemcpyDeviceToHost, h->stream);
        if (e != cudaSuccess) break;
        if (h->nscen > 1) {
            e = cudaMemcpyAsync(h->h_halt_bits, h->d_halt_bits,
                                sizeof(unsigned) * ((h->nscen + 31) / 32),
                                cudaMemcpyDeviceToHost, h->stream);
            if (e != cudaSuccess) break;
        }
        e = cudaEventRecord(ev[slot], h->stream);
        if (e != cudaSuccess) break;
        launched++;
        inflight++;
        slot ^= 1;
        if (inflight == 2) {
            e = cudaEventSynchronize(ev[slot]);  // the older of the two
            if (e != cudaSuccess) break;
            inflight--;
            if (h->h_summary->halted >= h->nscen || h->h_summary->status) halted = true;
            if (!halted && h->nscen > 1) {
                // ensembles: launch only up to the last scenario still running
                // (longest-running scenarios are placed first) once that
                // saves an eighth of the current launch
                int last = h->nscen - 1;
                while (last > 0 && (h->h_halt_bits[last >> 5] >> (last & 31) & 1u)) last--;
                const int extent = (int)h->scen_offsets[(size_t)last + 1];
                if (extent <= h->M.n_launch - h->M.n_launch / 8) {
                    e = cudaStreamSynchronize(h->stream);
                    if (e != cudaSuccess) break;
                    inflight = 0;
                    if ((rc = set_launch_extent(h, extent)) || (rc = build_graph(h))) {
                        cudaEventDestroy(ev[0]);
                        cudaEventDestroy(ev[1]);
                        cudaEventDestroy(t0);
                        cudaEventDestroy(t1);
                        return rc;
                    }
                }
            }
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(t1, h->stream);
    cudaError_t e2 = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess && elapsed_ms) {
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, t0, t1);
        *elapsed_ms = ms;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e != cudaSuccess) return fail(h, SWGPU_ECUDA, "evolve_run: %s", cudaGetErrorString(e));
    return finish_run(h, state);
}

int swgpu_evolve_one_step(void *handle, swgpu_state *state) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    int rc = prepare_run(h, 1);
    if (rc) return rc;
    if ((rc = issue_fused_step(h))) return rc;
    return finish_run(h, state);
}

int swgpu_synchronize(void *handle) {
    Handle *h = static_cast<Handle *>(handle);
    if (!h) return fail(h, SWGPU_EINVAL, "null handle");
    CK(cudaStreamSynchronize(h->stream));
    return SWGPU_OK;
}

}  // extern "C"

namespace swgpu {
Handle *handle_cast(void *p) { return static_cast<Handle *>(p); }
}  // namespace swgpu
