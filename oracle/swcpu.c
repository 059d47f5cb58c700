/*
 * swcpu.c -- CPU oracle for the ANUGA explicit shallow-water Euler step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain serial FP64 C, the
 * algorithm of the reference's ANUGA C path so that the CUDA library can be
 * checked against it.  Nothing in the product (libswgpu.so, the anuga_cuda
 * package) links, loads or calls this code; only tests/, the smoke check and
 * bench.py's CPU-baseline leg do.
 *
 * Layout follows ANUGA: triangle k, edge/vertex i live at [3*k + i]; normals
 * at [6*k + 2*i], coordinates at [6*k + 2*i] (x) and [6*k + 2*i + 1] (y).
 * Boundary edge m (neighbour index -m-1) has value slot m.
 *
 * Every routine names the reference file:line it follows (paths relative to
 * the reference project root).  Arithmetic is written so that each rounding
 * step happens in the same order as the reference: the file must be built
 * with -ffp-contract=off (no fused multiply-add), as the Makefile does.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "swcpu.h"

/* Sensitivity knob for tests: every pow and sin result of the oracle is
 * moved by libm_ulps units in the last place (0, the default, leaves them as
 * the host libm returns them).  A test sets it to measure how far a one-ulp
 * difference in a libm result -- CUDA's pow and sin against the host's --
 * carries through an evolve on its own. */
static int libm_ulps = 0;

void swcpu_set_libm_ulps(int n) { libm_ulps = n; }

static double libm_result(double x)
{
    int i;
    for (i = 0; i < libm_ulps; i++)
        x = nextafter(x, INFINITY);
    for (i = 0; i > libm_ulps; i--)
        x = nextafter(x, -INFINITY);
    return x;
}

/* src/anuga_HMPP/util_ext.h:45-59 -- max/min as plain comparisons (not
 * fmax/fmin): the result for equal or signed-zero arguments is the second
 * argument. */
static double omax(double x, double y) { return x > y ? x : y; }
static double omin(double x, double y) { return x < y ? x : y; }

/* ------------------------------------------------------------------ flux */

/* src/anuga_HMPP/shallow_water_ext.c:36-53 (_rotate). */
static void rotate3(double q[3], double n1, double n2)
{
    double a = q[1], b = q[2];
    q[1] = n1 * a + n2 * b;
    q[2] = -n2 * a + n1 * b;
}

/* src/anuga_HMPP/shallow_water_ext.c:214-242 (_compute_speed). */
static double limited_speed(double *uh, double *h, double eps, double h0,
                            double lim)
{
    double u;
    if (*h < lim) {
        if (*h < eps) {
            *h = 0.0;
            u = 0.0;
        } else {
            u = *uh / (*h + h0 / *h);
        }
        *uh = u * *h;
    } else {
        u = *uh / *h;
    }
    return u;
}

/* src/anuga_HMPP/shallow_water_ext.c:302-441 (_flux_function_central):
 * Kurganov-Noelle-Petrova central-upwind flux across one edge.  Returns 1 if
 * the bed is discontinuous across the edge (the reference reports an error
 * and returns with the flux untouched). */
static int central_flux(const double *ql, const double *qr, double zl,
                        double zr, double n1, double n2,
                        const swcpu_params *P, double h0, double lim,
                        double flux[3], double *max_speed)
{
    double L[3] = {ql[0], ql[1], ql[2]};
    double R[3] = {qr[0], qr[1], qr[2]};
    double fl[3], fr[3];
    double z, hl, hr, uhl, uhr, vhl, vhr, ul, ur, cl, cr, smax, smin, denom,
        inv;
    const double g = P->g, eps = P->epsilon;
    int i;

    rotate3(L, n1, n2);
    rotate3(R, n1, n2);

    if (fabs(zl - zr) > 1.0e-10)
        return 1;
    z = 0.5 * (zl + zr);

    hl = L[0] - z;
    uhl = L[1];
    ul = limited_speed(&uhl, &hl, eps, h0, lim);
    hr = R[0] - z;
    uhr = R[1];
    ur = limited_speed(&uhr, &hr, eps, h0, lim);

    vhl = L[2];
    vhr = R[2];
    limited_speed(&vhl, &hl, eps, h0, lim);
    limited_speed(&vhr, &hr, eps, h0, lim);

    cl = sqrt(g * hl);
    cr = sqrt(g * hr);

    smax = omax(ul + cl, ur + cr);
    if (smax < 0.0)
        smax = 0.0;
    smin = omin(ul - cl, ur - cr);
    if (smin > 0.0)
        smin = 0.0;

    fl[0] = ul * hl;
    fl[1] = ul * uhl + 0.5 * g * hl * hl;
    fl[2] = ul * vhl;
    fr[0] = ur * hr;
    fr[1] = ur * uhr + 0.5 * g * hr * hr;
    fr[2] = ur * vhr;

    denom = smax - smin;
    if (denom < eps) {
        flux[0] = flux[1] = flux[2] = 0.0;
        *max_speed = 0.0;
    } else {
        inv = 1.0 / denom;
        for (i = 0; i < 3; i++) {
            flux[i] = smax * fl[i] - smin * fr[i];
            flux[i] += smax * smin * (R[i] - L[i]);
            flux[i] *= inv;
        }
        *max_speed = omax(fabs(smax), fabs(smin));
        rotate3(flux, n1, -n2);
    }
    return 0;
}

/* src/anuga_HMPP/shallow_water_ext.c:4519-4696
 * (_compute_fluxes_central_structure): each edge is computed once, by the
 * first triangle that reaches it; the flux is subtracted from that triangle
 * and added to its neighbour.  Returns the CFL-limited flux timestep. */
double swcpu_compute_fluxes(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    const double h0 = P->H0 * P->H0;
    const double lim = 10 * P->H0;
    double timestep = P->evolve_max_timestep;
    double ql[3], qr[3], flux[3], zl, zr, ms, ms_total, length, inv_area;
    long k, n, m, ki, nm = 0;
    int i;
    unsigned char *done = D->work_flags;

    memset(D->stage_explicit_update, 0, N * sizeof(double));
    memset(D->xmom_explicit_update, 0, N * sizeof(double));
    memset(D->ymom_explicit_update, 0, N * sizeof(double));
    memset(done, 0, 3 * N);

    for (k = 0; k < N; k++) {
        ms_total = 0.0;
        for (i = 0; i < 3; i++) {
            ki = 3 * k + i;
            if (done[ki])
                continue;
            ql[0] = D->stage_edge_values[ki];
            ql[1] = D->xmom_edge_values[ki];
            ql[2] = D->ymom_edge_values[ki];
            zl = D->bed_edge_values[ki];
            n = D->neighbours[ki];
            if (n < 0) {
                m = -n - 1;
                qr[0] = D->stage_boundary_values[m];
                qr[1] = D->xmom_boundary_values[m];
                qr[2] = D->ymom_boundary_values[m];
                zr = zl;
            } else {
                m = D->neighbour_edges[ki];
                nm = 3 * n + m;
                qr[0] = D->stage_edge_values[nm];
                qr[1] = D->xmom_edge_values[nm];
                qr[2] = D->ymom_edge_values[nm];
                zr = D->bed_edge_values[nm];
            }
            if (P->optimise_dry_cells) {
                if (fabs(ql[0] - zl) < P->epsilon &&
                    fabs(qr[0] - zr) < P->epsilon) {
                    done[ki] = 1;
                    if (n >= 0)
                        done[nm] = 1;
                    continue;
                }
            }
            if (central_flux(ql, qr, zl, zr, D->normals[2 * ki],
                             D->normals[2 * ki + 1], P, h0, lim, flux, &ms)) {
                D->status |= SWCPU_ERR_DISCONTINUOUS_BED;
                return 0.0;
            }
            length = D->edgelengths[ki];
            flux[0] *= length;
            flux[1] *= length;
            flux[2] *= length;

            D->stage_explicit_update[k] -= flux[0];
            D->xmom_explicit_update[k] -= flux[1];
            D->ymom_explicit_update[k] -= flux[2];
            done[ki] = 1;
            if (n >= 0) {
                D->stage_explicit_update[n] += flux[0];
                D->xmom_explicit_update[n] += flux[1];
                D->ymom_explicit_update[n] += flux[2];
                done[nm] = 1;
            }
            if (D->tri_full_flag[k] == 1 && ms > P->epsilon) {
                timestep = omin(timestep, D->radii[k] / ms);
                if (n >= 0)
                    timestep = omin(timestep, D->radii[n] / ms);
            }
            ms_total = omax(ms_total, ms);
        }
        inv_area = 1.0 / D->areas[k];
        D->stage_explicit_update[k] *= inv_area;
        D->xmom_explicit_update[k] *= inv_area;
        D->ymom_explicit_update[k] *= inv_area;
        D->max_speed[k] = ms_total;
    }
    D->flux_timestep = timestep;
    return timestep;
}

/* The maximum wave speed of every edge evaluated from its own triangle's
 * side, triangle-centric (each interior edge twice, once from each of its
 * triangles), with the operations of swcpu_compute_fluxes: ms_out[3k + i],
 * or -1 where the dry-cell optimisation skips the edge.  Test support for
 * the timestep rule that lowers the timestep by each triangle's own radius
 * only.  Returns nonzero on a discontinuous bed. */
int swcpu_edge_speeds(const swcpu_domain *D, double *ms_out)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    const double h0 = P->H0 * P->H0;
    const double lim = 10 * P->H0;
    double ql[3], qr[3], flux[3], zl, zr, ms;
    long k, n, m, ki, nm;
    int i;

    for (k = 0; k < N; k++) {
        for (i = 0; i < 3; i++) {
            ki = 3 * k + i;
            ql[0] = D->stage_edge_values[ki];
            ql[1] = D->xmom_edge_values[ki];
            ql[2] = D->ymom_edge_values[ki];
            zl = D->bed_edge_values[ki];
            n = D->neighbours[ki];
            if (n < 0) {
                m = -n - 1;
                qr[0] = D->stage_boundary_values[m];
                qr[1] = D->xmom_boundary_values[m];
                qr[2] = D->ymom_boundary_values[m];
                zr = zl;
            } else {
                nm = 3 * n + D->neighbour_edges[ki];
                qr[0] = D->stage_edge_values[nm];
                qr[1] = D->xmom_edge_values[nm];
                qr[2] = D->ymom_edge_values[nm];
                zr = D->bed_edge_values[nm];
            }
            if (P->optimise_dry_cells && fabs(ql[0] - zl) < P->epsilon &&
                fabs(qr[0] - zr) < P->epsilon) {
                ms_out[ki] = -1.0;
                continue;
            }
            if (central_flux(ql, qr, zl, zr, D->normals[2 * ki], D->normals[2 * ki + 1], P,
                             h0, lim, flux, &ms))
                return 1;
            ms_out[ki] = ms;
        }
    }
    return 0;
}

/* src/anuga_HMPP/util_ext.h:66-108 (_gradient). */
static void plane_gradient(double x0, double y0, double x1, double y1,
                           double x2, double y2, double q0, double q1,
                           double q2, double *a, double *b)
{
    double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
    *a = (y2 - y0) * (q1 - q0) - (y1 - y0) * (q2 - q0);
    *a /= det;
    *b = (x1 - x0) * (q2 - q0) - (x2 - x0) * (q1 - q0);
    *b /= det;
}

/* src/anuga_HMPP/shallow_water_ext.c:1942-2036 (gravity_wb, loop body):
 * well-balanced gravity source -g h grad(w) plus the edge pressure side
 * term, added to the momentum explicit updates. */
void swcpu_gravity_wb(swcpu_domain *D)
{
    const double g = D->params->g;
    const long N = D->number_of_elements;
    long k;
    int i;
    for (k = 0; k < N; k++) {
        const long k3 = 3 * k, k6 = 6 * k;
        const double *X = D->vertex_coordinates + k6;
        double wx, wy, avg_h, hh[3], sidex = 0.0, sidey = 0.0, fact, area;
        plane_gradient(X[0], X[1], X[2], X[3], X[4], X[5],
                       D->stage_vertex_values[k3], D->stage_vertex_values[k3 + 1],
                       D->stage_vertex_values[k3 + 2], &wx, &wy);
        avg_h = D->stage_centroid_values[k] - D->bed_centroid_values[k];
        D->xmom_explicit_update[k] += -g * wx * avg_h;
        D->ymom_explicit_update[k] += -g * wy * avg_h;
        for (i = 0; i < 3; i++)
            hh[i] = D->stage_edge_values[k3 + i] - D->bed_edge_values[k3 + i];
        for (i = 0; i < 3; i++) {
            fact = -0.5 * g * hh[i] * hh[i] * D->edgelengths[k3 + i];
            sidex = sidex + fact * D->normals[k6 + 2 * i];
            sidey = sidey + fact * D->normals[k6 + 2 * i + 1];
        }
        area = D->areas[k];
        D->xmom_explicit_update[k] += -sidex / area;
        D->ymom_explicit_update[k] += -sidey / area;
    }
}

/* src/anuga_HMPP/shallow_water_ext.c:1238-1270 (_manning_friction_flat) and
 * :1272-1317 (_manning_friction_sloped): semi-implicit Manning friction,
 * eps = minimum_allowed_height as the reference GPU path passes it
 * (src/anuga_cuda/gpu_domain_advanced.py:1276-1318). */
static void manning_friction_into(swcpu_domain *D, double *xmom_update, double *ymom_update)
{
    const swcpu_params *P = D->params;
    const double g = P->g, eps = P->minimum_allowed_height;
    const long N = D->number_of_elements;
    long k;
    for (k = 0; k < N; k++) {
        const double eta = D->friction_centroid_values[k];
        const long k3 = 3 * k;
        double z0, z1, z2, z, h, S, zs = 1.0;
        if (!(eta > eps))
            continue;
        z0 = D->bed_vertex_values[k3];
        z1 = D->bed_vertex_values[k3 + 1];
        z2 = D->bed_vertex_values[k3 + 2];
        if (P->use_sloped_mannings) {
            const double *X = D->vertex_coordinates + 6 * k;
            double zx, zy;
            plane_gradient(X[0], X[1], X[2], X[3], X[4], X[5], z0, z1, z2, &zx,
                           &zy);
            zs = sqrt(1.0 + zx * zx + zy * zy);
        }
        z = (z0 + z1 + z2) / 3.0;
        h = D->stage_centroid_values[k] - z;
        if (h >= eps) {
            const double uh = D->xmom_centroid_values[k];
            const double vh = D->ymom_centroid_values[k];
            if (P->use_sloped_mannings)
                S = -g * eta * eta * zs * sqrt((uh * uh + vh * vh));
            else
                S = -g * eta * eta * sqrt((uh * uh + vh * vh));
            S /= libm_result(pow(h, 7.0 / 3));
            xmom_update[k] += S * uh;
            ymom_update[k] += S * vh;
        }
    }
}

/* manning_friction_implicit (gpu_domain_advanced.py:1255-1324): the term
 * goes to the semi-implicit updates. */
void swcpu_manning_friction(swcpu_domain *D)
{
    manning_friction_into(D, D->xmom_semi_implicit_update, D->ymom_semi_implicit_update);
}

/* manning_friction_explicit (gpu_domain_advanced.py:1330-1388): the same
 * kernels given the explicit updates. */
void swcpu_manning_friction_explicit(swcpu_domain *D)
{
    manning_friction_into(D, D->xmom_explicit_update, D->ymom_explicit_update);
}

/* src/anuga_HMPP/quantity.c:769-820 (_update) for one quantity.  Returns
 * nonzero if a semi-implicit denominator is not positive. */
static int update_one(long N, double dt, double *c, const double *expl,
                      double *semi)
{
    long k;
    double den;
    for (k = 0; k < N; k++) {
        if (c[k] == 0.0)
            semi[k] = 0.0;
        else
            semi[k] /= c[k];
    }
    for (k = 0; k < N; k++)
        c[k] += dt * expl[k];
    for (k = 0; k < N; k++) {
        den = 1.0 - dt * semi[k];
        if (den <= 0.0)
            return 1;
        c[k] /= den;
    }
    memset(semi, 0, N * sizeof(double));
    return 0;
}

/* src/anuga_cuda/gpu_domain_advanced.py:1412-1442
 * (update_conserved_quantities): _update for stage, xmom, ymom in turn. */
int swcpu_update_conserved_quantities(swcpu_domain *D, double dt)
{
    const long N = D->number_of_elements;
    int bad = 0;
    bad |= update_one(N, dt, D->stage_centroid_values, D->stage_explicit_update,
                      D->stage_semi_implicit_update);
    if (!bad)
        bad |= update_one(N, dt, D->xmom_centroid_values,
                          D->xmom_explicit_update, D->xmom_semi_implicit_update);
    if (!bad)
        bad |= update_one(N, dt, D->ymom_centroid_values,
                          D->ymom_explicit_update, D->ymom_semi_implicit_update);
    if (bad)
        D->status |= SWCPU_ERR_DENOMINATOR;
    return bad;
}

/* src/anuga_HMPP/shallow_water_ext.c:1638-1705 (_protect). */
void swcpu_protect(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    double *wc = D->stage_centroid_values, *uc = D->xmom_centroid_values,
           *vc = D->ymom_centroid_values;
    const double *zc = D->bed_centroid_values;
    long k;
    for (k = 0; k < N; k++) {
        const double hc = wc[k] - zc[k];
        if (!(hc < P->minimum_allowed_height))
            continue;
        if (P->maximum_allowed_speed < P->epsilon) {
            uc[k] = 0.0;
            vc[k] = 0.0;
            if (hc <= 0.0)
                wc[k] = zc[k];
        } else if (hc <= 0.0) {
            wc[k] = zc[k];
            uc[k] = 0.0;
            vc[k] = 0.0;
        } else {
            double u = uc[k] / hc, v = vc[k] / hc, r;
            if (fabs(u) > P->maximum_allowed_speed) {
                r = P->maximum_allowed_speed * u / fabs(u);
                uc[k] = r * hc;
            }
            if (fabs(v) > P->maximum_allowed_speed) {
                r = P->maximum_allowed_speed * v / fabs(v);
                vc[k] = r * hc;
            }
        }
    }
}

/* src/anuga_HMPP/shallow_water_ext.c:98-148 (find_qmin_and_qmax). */
static void qmin_qmax(double dq0, double dq1, double dq2, double *qmin,
                      double *qmax)
{
    if (dq0 >= 0.0) {
        if (dq1 >= dq2) {
            *qmax = (dq1 >= 0.0) ? dq0 + dq1 : dq0;
            *qmin = dq0 + dq2;
            if (*qmin >= 0.0)
                *qmin = 0.0;
        } else {
            *qmax = (dq2 > 0) ? dq0 + dq2 : dq0;
            *qmin = dq0 + dq1;
            if (*qmin >= 0.0)
                *qmin = 0.0;
        }
    } else {
        if (dq1 <= dq2) {
            *qmin = (dq1 < 0.0) ? dq0 + dq1 : dq0;
            *qmax = dq0 + dq2;
            if (*qmax <= 0.0)
                *qmax = 0.0;
        } else {
            *qmin = (dq2 < 0.0) ? dq0 + dq2 : dq0;
            *qmax = dq0 + dq1;
            if (*qmax <= 0.0)
                *qmax = 0.0;
        }
    }
}

/* src/anuga_HMPP/shallow_water_ext.c:151-181 (limit_gradient). */
static void limit_jumps(double dqv[3], double qmin, double qmax, double beta)
{
    const double TINY = 1.0e-100;
    double r = 1000.0, r0 = 1.0, phi;
    int i;
    for (i = 0; i < 3; i++) {
        if (dqv[i] < -TINY)
            r0 = qmin / dqv[i];
        if (dqv[i] > TINY)
            r0 = qmax / dqv[i];
        r = omin(r0, r);
    }
    phi = omin(r * beta, 1.0);
    dqv[0] = dqv[0] * phi;
    dqv[1] = dqv[1] * phi;
    dqv[2] = dqv[2] * phi;
}

/* Limited jumps of one quantity on the auxiliary triangle of three
 * surrogate-neighbour centroids (the per-quantity block repeated three times
 * in src/anuga_HMPP/shallow_water_ext.c:2942-3055). */
static void aux_triangle_jumps(double qk, double q0, double q1, double q2,
                               double dx1, double dy1, double dx2, double dy2,
                               double inv_area2, const double dxv[3],
                               const double dyv[3], double beta, double out[3])
{
    double dq0 = q0 - qk, dq1 = q1 - q0, dq2 = q2 - q0, a, b, qmin, qmax;
    double dqv[3];
    int i;
    a = dy2 * dq1 - dy1 * dq2;
    a *= inv_area2;
    b = dx1 * dq2 - dx2 * dq1;
    b *= inv_area2;
    for (i = 0; i < 3; i++)
        dqv[i] = a * dxv[i] + b * dyv[i];
    qmin_qmax(dq0, dq1, dq2, &qmin, &qmax);
    limit_jumps(dqv, qmin, qmax, beta);
    for (i = 0; i < 3; i++)
        out[i] = qk + dqv[i];
}

/* Limited jumps along the direction to the single interior neighbour
 * (src/anuga_HMPP/shallow_water_ext.c:3058-3205). */
static void one_neighbour_jumps(double qk, double q1, double dx2, double dy2,
                                const double dxv[3], const double dyv[3],
                                double beta, double out[3])
{
    double dq1 = q1 - qk, a = dq1 * dx2, b = dq1 * dy2, qmin, qmax, dqv[3];
    int i;
    for (i = 0; i < 3; i++)
        dqv[i] = a * dxv[i] + b * dyv[i];
    if (dq1 >= 0.0) {
        qmin = 0.0;
        qmax = dq1;
    } else {
        qmin = dq1;
        qmax = 0.0;
    }
    limit_jumps(dqv, qmin, qmax, beta);
    for (i = 0; i < 3; i++)
        out[i] = qk + dqv[i];
}

/* src/anuga_HMPP/shallow_water_ext.c:2717-3324
 * (_extrapolate_second_order_sw with the struct domain): limited
 * second-order reconstruction of stage and momentum (or velocity) at the
 * vertices.  Triangles whose surrogate neighbours are all dry keep their
 * previous vertex values; the velocity-to-momentum conversion at the end
 * applies to every triangle. */
void swcpu_extrapolate_second_order_sw(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    double *wc = D->stage_centroid_values, *zc = D->bed_centroid_values;
    double *uc = D->xmom_centroid_values, *vc = D->ymom_centroid_values;
    double *wv = D->stage_vertex_values, *uv = D->xmom_vertex_values,
           *vv = D->ymom_vertex_values;
    const double *zv = D->bed_vertex_values;
    const double *C = D->centroid_coordinates, *X = D->vertex_coordinates;
    double *ustore = D->work_a, *vstore = D->work_b;
    const int velocity = P->extrapolate_velocity_second_order == 1;
    long k;
    int i;

    if (velocity) {
        for (k = 0; k < N; k++) {
            double dk = omax(wc[k] - zc[k], P->minimum_allowed_height);
            ustore[k] = uc[k];
            uc[k] = uc[k] / dk;
            vstore[k] = vc[k];
            vc[k] = vc[k] / dk;
        }
    }

    for (k = 0; k < N; k++) {
        const long k3 = 3 * k, k6 = 6 * k;
        const long nb = D->number_of_boundaries[k];
        double x, y, dxv[3], dyv[3];
        if (nb == 3) {
            for (i = 0; i < 3; i++) {
                wv[k3 + i] = wc[k];
                uv[k3 + i] = uc[k];
                vv[k3 + i] = vc[k];
            }
            continue;
        }
        x = C[2 * k];
        y = C[2 * k + 1];
        for (i = 0; i < 3; i++) {
            dxv[i] = X[k6 + 2 * i] - x;
            dyv[i] = X[k6 + 2 * i + 1] - y;
        }
        if (nb <= 1) {
            const long k0 = D->surrogate_neighbours[k3];
            const long k1 = D->surrogate_neighbours[k3 + 1];
            const long k2 = D->surrogate_neighbours[k3 + 2];
            const double x0 = C[2 * k0], y0 = C[2 * k0 + 1];
            const double dx1 = C[2 * k1] - x0, dx2 = C[2 * k2] - x0;
            const double dy1 = C[2 * k1 + 1] - y0, dy2 = C[2 * k2 + 1] - y0;
            const double area2 = dy2 * dx1 - dy1 * dx2;
            double hc, h0, h1, h2, hmin, hfactor, inv_area2;
            if (area2 <= 0) {
                for (i = 0; i < 3; i++) {
                    wv[k3 + i] = wc[k];
                    uv[k3 + i] = uc[k];
                    vv[k3 + i] = vc[k];
                }
                continue;
            }
            hc = wc[k] - zc[k];
            h0 = wc[k0] - zc[k0];
            h1 = wc[k1] - zc[k1];
            h2 = wc[k2] - zc[k2];
            hmin = omin(omin(h0, omin(h1, h2)), hc);
            hfactor = 0.0;
            if (hmin > 0.001)
                hfactor = (hmin - 0.001) / (hmin + 0.004);
            if (P->optimise_dry_cells) {
                double hmax = omax(h0, omax(h1, h2));
                if (hmax < P->epsilon)
                    continue;
            }
            inv_area2 = 1.0 / area2;
            aux_triangle_jumps(wc[k], wc[k0], wc[k1], wc[k2], dx1, dy1, dx2,
                               dy2, inv_area2, dxv, dyv,
                               P->beta_w_dry + (P->beta_w - P->beta_w_dry) * hfactor,
                               wv + k3);
            aux_triangle_jumps(uc[k], uc[k0], uc[k1], uc[k2], dx1, dy1, dx2,
                               dy2, inv_area2, dxv, dyv,
                               P->beta_uh_dry + (P->beta_uh - P->beta_uh_dry) * hfactor,
                               uv + k3);
            aux_triangle_jumps(vc[k], vc[k0], vc[k1], vc[k2], dx1, dy1, dx2,
                               dy2, inv_area2, dxv, dyv,
                               P->beta_vh_dry + (P->beta_vh - P->beta_vh_dry) * hfactor,
                               vv + k3);
        } else {
            long j, k1 = -1;
            double dx1, dy1, area2, dx2, dy2;
            for (j = k3; j < k3 + 3; j++) {
                if (D->surrogate_neighbours[j] != k) {
                    k1 = D->surrogate_neighbours[j];
                    break;
                }
            }
            if (k1 < 0) {
                D->status |= SWCPU_ERR_NO_INTERIOR_NEIGHBOUR;
                return;
            }
            dx1 = C[2 * k1] - x;
            dy1 = C[2 * k1 + 1] - y;
            area2 = dx1 * dx1 + dy1 * dy1;
            dx2 = 1.0 / area2;
            dy2 = dx2 * dy1;
            dx2 *= dx1;
            one_neighbour_jumps(wc[k], wc[k1], dx2, dy2, dxv, dyv, P->beta_w,
                                wv + k3);
            one_neighbour_jumps(uc[k], uc[k1], dx2, dy2, dxv, dyv, P->beta_w,
                                uv + k3);
            one_neighbour_jumps(vc[k], vc[k1], dx2, dy2, dxv, dyv, P->beta_w,
                                vv + k3);
        }
    }

    if (velocity) {
        for (k = 0; k < N; k++) {
            const long k3 = 3 * k;
            for (i = 0; i < 3; i++) {
                double dv = omax(wv[k3 + i] - zv[k3 + i], 0.);
                uv[k3 + i] = uv[k3 + i] * dv;
                vv[k3 + i] = vv[k3 + i] * dv;
            }
            uc[k] = ustore[k];
            vc[k] = vstore[k];
        }
    }
}

/* src/anuga_cuda/extrapolate/extrapolate_first_order.cu:3-30: centroid
 * value copied to the three vertices (edges follow by interpolation). */
void swcpu_extrapolate_first_order(swcpu_domain *D)
{
    const long N = D->number_of_elements;
    long k;
    int i;
    for (k = 0; k < N; k++)
        for (i = 0; i < 3; i++) {
            D->stage_vertex_values[3 * k + i] = D->stage_centroid_values[k];
            D->xmom_vertex_values[3 * k + i] = D->xmom_centroid_values[k];
            D->ymom_vertex_values[3 * k + i] = D->ymom_centroid_values[k];
        }
}

/* src/anuga_HMPP/shallow_water_ext.c:1462-1636 (_balance_deep_and_shallow). */
void swcpu_balance_deep_and_shallow(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    const double eps = 1.0e-6;
    const double *wc = D->stage_centroid_values, *zc = D->bed_centroid_values;
    const double *uc = D->xmom_centroid_values, *vc = D->ymom_centroid_values;
    const double *zv = D->bed_vertex_values;
    double *wv = D->stage_vertex_values, *uv = D->xmom_vertex_values,
           *vv = D->ymom_vertex_values;
    long k;
    int i;
    for (k = 0; k < N; k++) {
        const long k3 = 3 * k;
        const double hc = wc[k] - zc[k];
        double dz = 0.0, hv[3], hmin, alpha, uu, vel;
        if (P->tight_slope_limiters == 0)
            for (i = 0; i < 3; i++)
                dz = omax(dz, fabs(zv[k3 + i] - zc[k]));
        for (i = 0; i < 3; i++)
            hv[i] = wv[k3 + i] - zv[k3 + i];
        hmin = omin(hv[0], omin(hv[1], hv[2]));
        if (P->tight_slope_limiters == 0) {
            if (dz > 0.0)
                alpha = omax(omin(P->alpha_balance * hmin / dz, 1.0), 0.0);
            else
                alpha = 1.0;
        } else if (hmin < P->H0) {
            alpha = 1.0;
            for (i = 0; i < 3; i++) {
                double hd = hc - hv[i];
                if (!(hd <= 0))
                    alpha = omin(alpha, (hc - P->H0) / hd);
            }
            if (alpha > 1.0)
                alpha = 1.0;
            if (alpha < 0.0)
                alpha = 0.0;
        } else {
            alpha = 1.0;
        }
        if (!(alpha < 1))
            continue;
        for (i = 0; i < 3; i++) {
            wv[k3 + i] = zv[k3 + i] + (1 - alpha) * hc + alpha * hv[i];
            if (P->use_centroid_velocities == 1) {
                if (hc > eps) {
                    uu = uc[k] / hc;
                    vel = vc[k] / hc;
                } else {
                    uu = 0.0;
                    vel = 0.0;
                }
                hv[i] = wv[k3 + i] - zv[k3 + i];
                uv[k3 + i] = uu * hv[i];
                vv[k3 + i] = vel * hv[i];
            } else {
                uv[k3 + i] = (1 - alpha) * uc[k] + alpha * uv[k3 + i];
                vv[k3 + i] = (1 - alpha) * vc[k] + alpha * vv[k3 + i];
            }
        }
    }
}

/* src/anuga_HMPP/quantity.c:687-706 (_interpolate_from_vertices_to_edges)
 * for stage, xmom and ymom. */
void swcpu_interpolate_to_edges(swcpu_domain *D)
{
    const long N = D->number_of_elements;
    double *V[3] = {D->stage_vertex_values, D->xmom_vertex_values,
                    D->ymom_vertex_values};
    double *E[3] = {D->stage_edge_values, D->xmom_edge_values,
                    D->ymom_edge_values};
    long k;
    int q;
    for (q = 0; q < 3; q++)
        for (k = 0; k < N; k++) {
            const double q0 = V[q][3 * k], q1 = V[q][3 * k + 1],
                         q2 = V[q][3 * k + 2];
            E[q][3 * k] = 0.5 * (q1 + q2);
            E[q][3 * k + 1] = 0.5 * (q0 + q2);
            E[q][3 * k + 2] = 0.5 * (q0 + q1);
        }
}

/* src/anuga_cuda/gpu_domain_advanced.py:1884-1986: protect, then first- or
 * second-order extrapolation, balance, and vertex-to-edge interpolation. */
/* Gradient of the plane through three points, src/anuga_HMPP/util_ext.h:66-108. */
static void gradient3(double x0, double y0, double x1, double y1, double x2, double y2,
                      double q0, double q1, double q2, double *a, double *b)
{
    const double det = (y2 - y0) * (x1 - x0) - (y1 - y0) * (x2 - x0);
    *a = (y2 - y0) * (q1 - q0) - (y1 - y0) * (q2 - q0);
    *a /= det;
    *b = (x1 - x0) * (q2 - q0) - (x2 - x0) * (q1 - q0);
    *b /= det;
}

/* Two-point gradient, constant across the line, util_ext.h:111-162. */
static void gradient2(double x0, double y0, double x1, double y1, double q0, double q1,
                      double *a, double *b)
{
    const double xx = x1 - x0, yy = y1 - y0, qq = q1 - q0;
    const double det = xx * xx + yy * yy;
    *a = xx * qq / det;
    *b = yy * qq / det;
}

/* Quantity.extrapolate_second_order_and_limit_by_vertex / _by_edge for one
 * quantity: _compute_gradients (src/anuga_HMPP/quantity.c:24-95; no true
 * neighbour leaves the gradient at zero), _extrapolate_from_gradient
 * (:130-172) and _limit_vertices_by_all_neighbours (:298-361) or
 * _limit_edges_by_all_neighbours (:363-447).  Writes vertex and edge values.
 * Returns nonzero where _compute_gradients would stop (repeated surrogate). */
static int limit_one_quantity(const swcpu_domain *D, const double *qc, double *qv, double *qe,
                              double beta, int by_edge)
{
    const long N = D->number_of_elements;
    const double *C = D->centroid_coordinates, *X = D->vertex_coordinates;
    long k;
    int i, err = 0;
    for (k = 0; k < N; k++) {
        const long *s = D->surrogate_neighbours + 3 * k;
        const long nb = D->number_of_boundaries[k];
        double a = 0.0, b = 0.0, v[3], e[3], dqa[3], qmin, qmax, phi = 1.0;
        const double q = qc[k], x = C[2 * k], y = C[2 * k + 1];
        if (nb < 2) {
            if (s[0] == s[1] || s[1] == s[2]) {
                err = 1;
            } else {
                gradient3(C[2 * s[0]], C[2 * s[0] + 1], C[2 * s[1]], C[2 * s[1] + 1],
                          C[2 * s[2]], C[2 * s[2] + 1], qc[s[0]], qc[s[1]], qc[s[2]], &a, &b);
            }
        } else if (nb == 2) {
            long k0 = k;
            for (i = 0; i < 3 && k0 == k; i++)
                k0 = s[i];
            if (k0 == k)
                err = 1;
            else
                gradient2(C[2 * k0], C[2 * k0 + 1], x, y, qc[k0], q, &a, &b);
        }
        for (i = 0; i < 3; i++)
            v[i] = q + a * (X[6 * k + 2 * i] - x) + b * (X[6 * k + 2 * i + 1] - y);
        e[0] = 0.5 * (v[1] + v[2]);
        e[1] = 0.5 * (v[2] + v[0]);
        e[2] = 0.5 * (v[0] + v[1]);
        qmin = qmax = q;
        for (i = 0; i < 3; i++) {
            const long n = D->neighbours[3 * k + i];
            if (n >= 0) {
                qmin = omin(qmin, qc[n]);
                qmax = omax(qmax, qc[n]);
            }
        }
        for (i = 0; i < 3; i++) {
            double r = 1.0;
            const double dq = (by_edge ? e[i] : v[i]) - q;
            dqa[i] = dq;
            if (dq > 0.0)
                r = (qmax - q) / dq;
            if (dq < 0.0)
                r = (qmin - q) / dq;
            phi = omin(omin(r * beta, 1.0), phi);
        }
        if (by_edge) {
            for (i = 0; i < 3; i++)
                e[i] = q + phi * dqa[i];
            v[0] = e[1] + e[2] - e[0];
            v[1] = e[2] + e[0] - e[1];
            v[2] = e[0] + e[1] - e[2];
        } else {
            for (i = 0; i < 3; i++)
                v[i] = q + phi * dqa[i];
            e[0] = 0.5 * (v[1] + v[2]);
            e[1] = 0.5 * (v[2] + v[0]);
            e[2] = 0.5 * (v[0] + v[1]);
        }
        for (i = 0; i < 3; i++) {
            qv[3 * k + i] = v[i];
            qe[3 * k + i] = e[i];
        }
    }
    return err;
}

/* The per-quantity limiter branch of distribute_to_vertices_and_edges
 * (src/anuga_cuda/gpu_domain_advanced.py:1815-1860 by edge, :1918-1943 by
 * vertex): stage, xmomentum and ymomentum each with its own beta. */
int swcpu_extrapolate_and_limit_by_neighbours(swcpu_domain *D, int by_edge)
{
    const swcpu_params *P = D->params;
    int err = 0;
    err |= limit_one_quantity(D, D->stage_centroid_values, D->stage_vertex_values,
                              D->stage_edge_values, P->beta_w, by_edge);
    err |= limit_one_quantity(D, D->xmom_centroid_values, D->xmom_vertex_values,
                              D->xmom_edge_values, P->beta_uh, by_edge);
    err |= limit_one_quantity(D, D->ymom_centroid_values, D->ymom_vertex_values,
                              D->ymom_edge_values, P->beta_vh, by_edge);
    if (err)
        D->status |= SWCPU_ERR_NO_INTERIOR_NEIGHBOUR;
    return err;
}

/* The 'tsunami' protection, src/anuga_cuda/protect/protect.cu:64-131
 * (_protect_swb2; HMPP restatement src/anuga_HMPP/swb2_domain_ext.c:7-79):
 * below max(0.1 (max bed edge - bed centroid), minimum_allowed_height)
 * momentum is zeroed; a non-positive depth lifts stage (and the stage
 * vertex values) to the lowest bed vertex minus minimum_allowed_height. */
void swcpu_protect_swb2(swcpu_domain *D)
{
    const double mah = D->params->minimum_allowed_height;
    const double minimum_relative_height = 0.1;
    double *wc = D->stage_centroid_values, *wv = D->stage_vertex_values;
    const double *zc = D->bed_centroid_values, *zv = D->bed_vertex_values;
    long k;
    for (k = 0; k < D->number_of_elements; k++) {
        const double hc = wc[k] - zc[k];
        const double bmax = 0.5 * fmax(zv[3 * k] + zv[3 * k + 1],
                                       fmax(zv[3 * k + 1] + zv[3 * k + 2],
                                            zv[3 * k + 2] + zv[3 * k]));
        if (hc < fmax(minimum_relative_height * (bmax - zc[k]), mah)) {
            D->xmom_centroid_values[k] = 0.0;
            D->ymom_centroid_values[k] = 0.0;
            if (hc <= 0.0) {
                const double bmin = fmin(zv[3 * k], fmin(zv[3 * k + 1], zv[3 * k + 2])) - mah;
                if (wc[k] < bmin) {
                    wc[k] = fmax(wc[k], bmin);
                    wv[3 * k] = fmax(wv[3 * k], bmin);
                    wv[3 * k + 1] = fmax(wv[3 * k + 1], bmin);
                    wv[3 * k + 2] = fmax(wv[3 * k + 2], bmin);
                }
            }
        }
    }
}

/* The limiter of the edge extrapolation: src/anuga_HMPP/
 * shallow_water_ext.c:151-180 (limit_gradient) applied to edge jumps. */
static void limit_gradient_jumps(double dqv[3], double qmin, double qmax, double beta)
{
    const double tiny = 1.0e-100;
    double r = 1000.0, r0 = 1.0, phi;
    int i;
    for (i = 0; i < 3; i++) {
        if (dqv[i] < -tiny)
            r0 = qmin / dqv[i];
        if (dqv[i] > tiny)
            r0 = qmax / dqv[i];
        r = omin(r0, r);
    }
    phi = omin(r * beta, 1.0);
    dqv[0] = dqv[0] * phi;
    dqv[1] = dqv[1] * phi;
    dqv[2] = dqv[2] * phi;
}

/* src/anuga_HMPP/shallow_water_ext.c:3328-3964 (_extrapolate_second_order_edge_sw),
 * the extrapolation of the 'tsunami' algorithm: limited gradients as in
 * extrapolate_second_order_sw but evaluated at the edge midpoints, dry
 * surrogate neighbours replaced by the triangle itself, beta switched fully
 * wet/dry (hfactor 0 or 1), vertex values from the edge values
 * (v_i = e_j + e_k - e_i), velocities converted back to momenta with the
 * edge and vertex depths.  Cells skipped as dry keep their previous edge
 * values (and, as in the reference, rescale them by depth). */
int swcpu_extrapolate_second_order_edge_sw(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    const long N = D->number_of_elements;
    const double *C = D->centroid_coordinates, *E = D->edge_coordinates;
    const double *w = D->stage_centroid_values, *z = D->bed_centroid_values;
    double *we = D->stage_edge_values, *ue = D->xmom_edge_values, *ve = D->ymom_edge_values;
    double *u = D->work_a, *v = D->work_b;  /* momentum or velocity at centroids */
    const int vel = P->extrapolate_velocity_second_order == 1;
    long k;
    int i, err = 0;
    for (k = 0; k < N; k++) {
        if (vel) {
            const double dk = omax(w[k] - z[k], P->minimum_allowed_height);
            u[k] = D->xmom_centroid_values[k] / dk;
            v[k] = D->ymom_centroid_values[k] / dk;
        } else {
            u[k] = D->xmom_centroid_values[k];
            v[k] = D->ymom_centroid_values[k];
        }
    }
    for (k = 0; k < N; k++) {
        const long k3 = 3 * k, k6 = 6 * k;
        const long nb = D->number_of_boundaries[k];
        double dxv[3], dyv[3], dqv[3], qmin, qmax;
        const double x = C[2 * k], y = C[2 * k + 1];
        if (nb == 3) {
            for (i = 0; i < 3; i++) {
                we[k3 + i] = w[k];
                ue[k3 + i] = u[k];
                ve[k3 + i] = v[k];
            }
            continue;
        }
        for (i = 0; i < 3; i++) {
            dxv[i] = E[k6 + 2 * i] - x;
            dyv[i] = E[k6 + 2 * i + 1] - y;
        }
        if (nb <= 1) {
            long k0 = D->surrogate_neighbours[k3], k1 = D->surrogate_neighbours[k3 + 1];
            long k2 = D->surrogate_neighbours[k3 + 2];
            double x0, y0, dx1, dx2, dy1, dy2, area2, inv_area2, hc, h0, h1, h2, hmin, hfactor;
            const double *q[3];
            double *qe[3];
            double beta[3];
            int j;
            if (w[k2] <= z[k2])
                k2 = k;
            if (w[k0] <= z[k0])
                k0 = k;
            if (w[k1] <= z[k1])
                k1 = k;
            x0 = C[2 * k0];
            y0 = C[2 * k0 + 1];
            dx1 = C[2 * k1] - x0;
            dx2 = C[2 * k2] - x0;
            dy1 = C[2 * k1 + 1] - y0;
            dy2 = C[2 * k2 + 1] - y0;
            area2 = dy2 * dx1 - dy1 * dx2;
            if (area2 <= 0) {
                for (i = 0; i < 3; i++) {
                    we[k3 + i] = w[k];
                    ue[k3 + i] = u[k];
                    ve[k3 + i] = v[k];
                }
                continue;
            }
            hc = w[k] - z[k];
            h0 = w[k0] - z[k0];
            h1 = w[k1] - z[k1];
            h2 = w[k2] - z[k2];
            hmin = omin(omin(h0, omin(h1, h2)), hc);
            hfactor = hmin > 0.0 ? 1.0 : 0.0;
            if (P->optimise_dry_cells && omax(h0, omax(h1, h2)) < P->epsilon)
                continue;
            inv_area2 = 1.0 / area2;
            q[0] = w;
            q[1] = u;
            q[2] = v;
            qe[0] = we;
            qe[1] = ue;
            qe[2] = ve;
            beta[0] = P->beta_w_dry + (P->beta_w - P->beta_w_dry) * hfactor;
            beta[1] = P->beta_uh_dry + (P->beta_uh - P->beta_uh_dry) * hfactor;
            beta[2] = P->beta_vh_dry + (P->beta_vh - P->beta_vh_dry) * hfactor;
            for (j = 0; j < 3; j++) {
                const double dq0 = q[j][k0] - q[j][k];
                const double dq1 = q[j][k1] - q[j][k0];
                const double dq2 = q[j][k2] - q[j][k0];
                double a = dy2 * dq1 - dy1 * dq2, b = dx1 * dq2 - dx2 * dq1;
                a *= inv_area2;
                b *= inv_area2;
                for (i = 0; i < 3; i++)
                    dqv[i] = a * dxv[i] + b * dyv[i];
                qmin_qmax(dq0, dq1, dq2, &qmin, &qmax);
                limit_gradient_jumps(dqv, qmin, qmax, beta[j]);
                for (i = 0; i < 3; i++)
                    qe[j][k3 + i] = q[j][k] + dqv[i];
            }
        } else {
            /* one interior neighbour: the first surrogate that is not k */
            long k1 = -1;
            double dx1, dy1, area2, dx2, dy2;
            const double *q[3];
            double *qe[3];
            int j;
            for (i = 0; i < 3; i++)
                if (D->surrogate_neighbours[k3 + i] != k) {
                    k1 = D->surrogate_neighbours[k3 + i];
                    break;
                }
            if (k1 < 0) {
                err = 1;
                continue;
            }
            dx1 = C[2 * k1] - x;
            dy1 = C[2 * k1 + 1] - y;
            area2 = dx1 * dx1 + dy1 * dy1;
            dx2 = 1.0 / area2;
            dy2 = dx2 * dy1;
            dx2 *= dx1;
            q[0] = w;
            q[1] = u;
            q[2] = v;
            qe[0] = we;
            qe[1] = ue;
            qe[2] = ve;
            for (j = 0; j < 3; j++) {
                const double dq1 = q[j][k1] - q[j][k];
                const double a = dq1 * dx2, b = dq1 * dy2;
                for (i = 0; i < 3; i++)
                    dqv[i] = a * dxv[i] + b * dyv[i];
                if (dq1 >= 0.0) {
                    qmin = 0.0;
                    qmax = dq1;
                } else {
                    qmin = dq1;
                    qmax = 0.0;
                }
                limit_gradient_jumps(dqv, qmin, qmax, P->beta_w);
                for (i = 0; i < 3; i++)
                    qe[j][k3 + i] = q[j][k] + dqv[i];
            }
        }
    }
    for (k = 0; k < N; k++) {
        const long k3 = 3 * k;
        double *qv[3] = {D->stage_vertex_values, D->xmom_vertex_values, D->ymom_vertex_values};
        double *qe[3] = {we, ue, ve};
        int j;
        for (j = 0; j < 3; j++) {
            qv[j][k3] = qe[j][k3 + 1] + qe[j][k3 + 2] - qe[j][k3];
            qv[j][k3 + 1] = qe[j][k3] + qe[j][k3 + 2] - qe[j][k3 + 1];
            qv[j][k3 + 2] = qe[j][k3] + qe[j][k3 + 1] - qe[j][k3 + 2];
        }
        if (vel) {
            for (i = 0; i < 3; i++) {
                const double de = omax(we[k3 + i] - D->bed_edge_values[k3 + i], 0.0);
                ue[k3 + i] = ue[k3 + i] * de;
                ve[k3 + i] = ve[k3 + i] * de;
            }
            for (i = 0; i < 3; i++) {
                const double dv = omax(D->stage_vertex_values[k3 + i] -
                                           D->bed_vertex_values[k3 + i], 0.0);
                D->xmom_vertex_values[k3 + i] = D->xmom_vertex_values[k3 + i] * dv;
                D->ymom_vertex_values[k3 + i] = D->ymom_vertex_values[k3 + i] * dv;
            }
        }
    }
    if (err)
        D->status |= SWCPU_ERR_NO_INTERIOR_NEIGHBOUR;
    return err;
}

/* src/anuga_cuda/gpu_domain_advanced.py:1744-2001: protect, then first
 * order, the per-quantity edge limiter (use_edge_limiter), the optimised
 * shallow-water extrapolation (optimised_gradient_limiter) or the
 * per-quantity vertex limiter; then balance and edge interpolation. */
void swcpu_distribute_to_vertices_and_edges(swcpu_domain *D)
{
    const swcpu_params *P = D->params;
    if (P->flow_algorithm == 1) {
        /* the 'tsunami' branch (:1755-1812): protect_swb2 and the edge
         * extrapolation, at every order, no balance */
        swcpu_protect_swb2(D);
        swcpu_extrapolate_second_order_edge_sw(D);
        return;
    }
    swcpu_protect(D);
    if (D->order == 1)
        swcpu_extrapolate_first_order(D);
    else if (P->use_edge_limiter)
        swcpu_extrapolate_and_limit_by_neighbours(D, 1);
    else if (P->optimised_gradient_limiter)
        swcpu_extrapolate_second_order_sw(D);
    else
        swcpu_extrapolate_and_limit_by_neighbours(D, 0);
    swcpu_balance_deep_and_shallow(D);
    swcpu_interpolate_to_edges(D);
}

/* ------------------------------------------------------------- boundary */

/* Boundary conditions, one value slot per boundary edge.
 * Reflective: src/anuga_cuda/evaluate_segment/evaluate_segment.cu:3-76
 * (edge stage copied, momentum mirrored about the edge normal).
 * Dirichlet: evaluate_segment.cu:80-115 (edge values copied, then the
 * conserved quantities set to constants).
 * Time-dependent stage (no reference GPU counterpart: the reference raises
 * for any other boundary type, gpu_domain_advanced.py:2099-2100):
 * stage = mean + amplitude*sin(2*pi*t/period + phase), momentum 0, evaluated
 * at the model time when update_boundary runs. */
/* Unit discharge of a triangular hydrograph with parameters (peak, rise,
 * fall, start): 0 before start, linear to peak over rise, linear to 0 over
 * fall, then 0. */
double swcpu_hydrograph(const double p[4], double t)
{
    const double s = t - p[3];
    if (s <= 0.0)
        return 0.0;
    if (s < p[1])
        return p[0] * (s / p[1]);
    if (s < p[1] + p[2])
        return p[0] * (1.0 - (s - p[1]) / p[2]);
    return 0.0;
}

void swcpu_update_boundary(swcpu_domain *D)
{
    const long Nb = D->number_of_boundary_elements;
    long m;
    for (m = 0; m < Nb; m++) {
        const long vol = D->boundary_cells[m], e = D->boundary_edges[m];
        const long ki = 3 * vol + e;
        const swcpu_boundary_tag *T = &D->tags[D->boundary_tag[m]];
        D->bed_boundary_values[m] = D->bed_edge_values[ki];
        if (T->type == SWCPU_BC_REFLECTIVE) {
            const double n1 = D->normals[2 * ki], n2 = D->normals[2 * ki + 1];
            const double q1 = D->xmom_edge_values[ki], q2 = D->ymom_edge_values[ki];
            const double r1 = -q1 * n1 - q2 * n2;
            const double r2 = -q1 * n2 + q2 * n1;
            D->stage_boundary_values[m] = D->stage_edge_values[ki];
            D->xmom_boundary_values[m] = n1 * r1 - n2 * r2;
            D->ymom_boundary_values[m] = n2 * r1 + n1 * r2;
        } else if (T->type == SWCPU_BC_DIRICHLET) {
            D->stage_boundary_values[m] = T->p[0];
            D->xmom_boundary_values[m] = T->p[1];
            D->ymom_boundary_values[m] = T->p[2];
        } else if (T->type == SWCPU_BC_TIME_STAGE_SINE) {
            const double two_pi = 6.283185307179586;
            D->stage_boundary_values[m] =
                T->p[0] + T->p[1] * libm_result(sin(two_pi * D->time / T->p[2] + T->p[3]));
            D->xmom_boundary_values[m] = 0.0;
            D->ymom_boundary_values[m] = 0.0;
        } else if (T->type == SWCPU_BC_TIME_STAGE_FOURIER) {
            /* an ANUGA Time_boundary whose function is the truncated
             * Fourier series c0 + c1 sin(wt) + c2 cos(wt) + c3 sin(2wt) +
             * c4 cos(2wt), w = 2 pi / period, with zero momentum */
            const double wt = 6.283185307179586 * D->time / T->p[5];
            D->stage_boundary_values[m] =
                T->p[0] + T->p[1] * libm_result(sin(wt)) + T->p[2] * libm_result(cos(wt)) +
                T->p[3] * libm_result(sin(2.0 * wt)) + T->p[4] * libm_result(cos(2.0 * wt));
            D->xmom_boundary_values[m] = 0.0;
            D->ymom_boundary_values[m] = 0.0;
        } else if (T->type == SWCPU_BC_TRANSMISSIVE) {
            /* anuga Transmissive_boundary: the inside edge values */
            D->stage_boundary_values[m] = D->stage_edge_values[ki];
            D->xmom_boundary_values[m] = D->xmom_edge_values[ki];
            D->ymom_boundary_values[m] = D->ymom_edge_values[ki];
        } else if (T->type == SWCPU_BC_TRANSMISSIVE_STAGE_ZERO_MOMENTUM) {
            /* anuga Transmissive_stage_zero_momentum_boundary */
            D->stage_boundary_values[m] = D->stage_edge_values[ki];
            D->xmom_boundary_values[m] = 0.0;
            D->ymom_boundary_values[m] = 0.0;
        } else if (T->type == SWCPU_BC_INFLOW_HYDROGRAPH) {
            /* triangular hydrograph of unit discharge q(t) entering through
             * the edge: stage the inside edge's, or critical depth
             * (q^2/g)^(1/3) above the edge bed where that is higher */
            const double q = swcpu_hydrograph(T->p, D->time);
            const double h = cbrt(q * q / D->params->g);
            const double n1 = D->normals[2 * ki], n2 = D->normals[2 * ki + 1];
            D->stage_boundary_values[m] = omax(D->stage_edge_values[ki], D->bed_edge_values[ki] + h);
            D->xmom_boundary_values[m] = -q * n1;
            D->ymom_boundary_values[m] = -q * n2;
        } else {
            D->status |= SWCPU_ERR_BOUNDARY_TYPE;
        }
    }
}

/* ---------------------------------------------------------- time stepping */

/* ANUGA Generic_Domain.update_timestep as restated in
 * src/anuga_HMPP/evolve.c:115-160, with the finaltime clamp written as
 * finaltime - time (evolve.c:147-148 adds them).  finaltime <= 0 means none. */
void swcpu_update_timestep(swcpu_domain *D, double finaltime)
{
    const swcpu_params *P = D->params;
    double dt = omin(P->CFL * D->flux_timestep, P->evolve_max_timestep);
    D->recorded_max_timestep = omax(dt, D->recorded_max_timestep);
    D->recorded_min_timestep = omin(dt, D->recorded_min_timestep);
    if (dt < P->evolve_min_timestep) {
        D->smallsteps += 1;
        if (D->smallsteps > P->max_smallsteps) {
            D->smallsteps = 0;
            if (D->order == 1) {
                dt = P->evolve_min_timestep;
                D->status |= SWCPU_ERR_SMALL_TIMESTEP;
            } else {
                D->order = 1;
            }
        }
    } else {
        D->smallsteps = 0;
        if (D->order == 1 && P->default_order == 2)
            D->order = 2;
    }
    if (finaltime > 0 && D->time + dt > finaltime)
        dt = finaltime - D->time;
    if (D->time + dt > D->yieldtime)
        dt = D->yieldtime - D->time;
    D->timestep = dt;
}

/* src/anuga_cuda/gpu_domain_advanced.py:2178-2191 (evolve_one_euler_step):
 * fluxes with the gravity term (compute_fluxes_method 'wb_2'), Manning
 * friction, timestep, conserved update. */
int swcpu_evolve_one_euler_step(swcpu_domain *D, double finaltime)
{
    swcpu_compute_fluxes(D);
    swcpu_gravity_wb(D);
    swcpu_manning_friction(D);
    swcpu_update_timestep(D, finaltime);
    swcpu_update_conserved_quantities(D, D->timestep);
    return D->status;
}

/* src/anuga_cuda/gpu_domain_advanced.py:1449-1478 (backup_conserved_quantities):
 * centroid copies of stage, xmomentum and ymomentum. */
void swcpu_backup_conserved_quantities(swcpu_domain *D)
{
    long k;
    for (k = 0; k < D->number_of_elements; k++) {
        D->stage_centroid_backup[k] = D->stage_centroid_values[k];
        D->xmom_centroid_backup[k] = D->xmom_centroid_values[k];
        D->ymom_centroid_backup[k] = D->ymom_centroid_values[k];
    }
}

/* src/anuga_HMPP/quantity.c:749-765 (_saxpy_centroid_values), applied to the
 * three conserved quantities (gpu_domain_advanced.py:1484-1519):
 * Q = a*Q + b*backup, two products and one sum, no contraction. */
void swcpu_saxpy_conserved_quantities(swcpu_domain *D, double a, double b)
{
    double *q[3] = {D->stage_centroid_values, D->xmom_centroid_values,
                    D->ymom_centroid_values};
    const double *qb[3] = {D->stage_centroid_backup, D->xmom_centroid_backup,
                           D->ymom_centroid_backup};
    long k;
    int i;
    for (i = 0; i < 3; i++)
        for (k = 0; k < D->number_of_elements; k++)
            q[i][k] = a * q[i][k] + b * qb[i][k];
}

/* One forward-Euler stage with the step's timestep already chosen: fluxes,
 * forcing (gravity_wb and Manning friction), conserved update. */
static int rk_stage(swcpu_domain *D)
{
    swcpu_compute_fluxes(D);
    swcpu_gravity_wb(D);
    swcpu_manning_friction(D);
    swcpu_update_conserved_quantities(D, D->timestep);
    return (int)D->status;
}

/* ANUGA Generic_Domain.evolve_one_rk2_step (anuga_core generic_domain.py;
 * ANUGA is a dependency that the reference does not vendor, called at
 * src/anuga_cuda/gpu_domain_advanced.py:2198-2204 and :2569-2570):
 *   Q^{n+1} = 1/2 Q^n + 1/2 E(h)^2 Q^n
 * backup; Euler stage with update_timestep; time += dt; distribute and
 * boundaries; second Euler stage with the same dt; saxpy(1/2, 1/2).  The
 * evolve loop then sets time = t0 + dt and distributes. */
int swcpu_evolve_one_rk2_step(swcpu_domain *D, double finaltime)
{
    swcpu_backup_conserved_quantities(D);
    if (swcpu_evolve_one_euler_step(D, finaltime))
        return (int)D->status;
    D->time = D->time + D->timestep;
    swcpu_distribute_to_vertices_and_edges(D);
    swcpu_update_boundary(D);
    if (rk_stage(D))
        return (int)D->status;
    swcpu_saxpy_conserved_quantities(D, 0.5, 0.5);
    return (int)D->status;
}

/* ANUGA Generic_Domain.evolve_one_rk3_step (same dependency; called at
 * src/anuga_cuda/gpu_domain_advanced.py:2248-2254 and :2572-2573), the
 * three-stage strong-stability-preserving scheme:
 *   Q1 = E(h) Q^n;  Q2 = 3/4 Q^n + 1/4 E(h) Q1 at t0 + h/2;
 *   Q^{n+1} = 1/3 Q^n + 2/3 E(h) Q2,
 * every stage with the dt chosen by the first. */
int swcpu_evolve_one_rk3_step(swcpu_domain *D, double finaltime)
{
    const double t0 = D->time;
    swcpu_backup_conserved_quantities(D);
    if (swcpu_evolve_one_euler_step(D, finaltime))
        return (int)D->status;
    D->time = D->time + D->timestep;
    swcpu_distribute_to_vertices_and_edges(D);
    swcpu_update_boundary(D);
    if (rk_stage(D))
        return (int)D->status;
    swcpu_saxpy_conserved_quantities(D, 0.25, 0.75);
    D->time = t0 + D->timestep * 0.5;
    swcpu_distribute_to_vertices_and_edges(D);
    swcpu_update_boundary(D);
    if (rk_stage(D))
        return (int)D->status;
    swcpu_saxpy_conserved_quantities(D, 2.0 / 3.0, 1.0 / 3.0);
    return (int)D->status;
}

/* The set-up half of src/anuga_cuda/gpu_domain_advanced.py:2476-2551:
 * distribute, reset time and counters, distribute again, boundaries. */
void swcpu_evolve_start(swcpu_domain *D, double yieldstep)
{
    swcpu_distribute_to_vertices_and_edges(D);
    D->time = D->starttime;
    D->order = D->params->default_order;
    D->yieldtime = D->time + yieldstep;
    D->recorded_min_timestep = D->params->evolve_max_timestep;
    D->recorded_max_timestep = D->params->evolve_min_timestep;
    D->number_of_steps = 0;
    D->smallsteps = 0;
    swcpu_distribute_to_vertices_and_edges(D);
    swcpu_update_boundary(D);
}

/* One pass of the hot loop of src/anuga_cuda/gpu_domain_advanced.py:2555-2675
 * until the next yield point, the final time, or max_steps steps.  Returns
 * 1 at a yield point, 2 at the final time, 0 when max_steps ran out, and a
 * negative value on error.  The caller advances yieldtime after a yield. */
int swcpu_evolve_steps(swcpu_domain *D, double yieldstep, double finaltime,
                       long max_steps, double time_epsilon)
{
    long s;
    for (s = 0; s < max_steps; s++) {
        const double t0 = D->time;
        if (D->timestepping_method == 2)
            swcpu_evolve_one_rk2_step(D, finaltime);
        else if (D->timestepping_method == 3)
            swcpu_evolve_one_rk3_step(D, finaltime);
        else
            swcpu_evolve_one_euler_step(D, finaltime);
        if (D->status)
            return -1;
        D->time = t0 + D->timestep;
        swcpu_distribute_to_vertices_and_edges(D);
        swcpu_update_boundary(D);
        D->number_of_steps += 1;
        if (D->status)
            return -1;
        if (finaltime > 0 && D->time >= finaltime - time_epsilon) {
            D->time = finaltime;
            return 2;
        }
        if (D->time >= D->yieldtime) {
            D->yieldtime += yieldstep;
            D->recorded_min_timestep = D->params->evolve_max_timestep;
            D->recorded_max_timestep = D->params->evolve_min_timestep;
            D->number_of_steps = 0;
            return 1;
        }
    }
    return 0;
}

/* Total water volume sum(area * (stage - bed)) in triangle order. */
double swcpu_mass(const swcpu_domain *D)
{
    double s = 0.0;
    long k;
    for (k = 0; k < D->number_of_elements; k++)
        s += D->areas[k] *
             (D->stage_centroid_values[k] - D->bed_centroid_values[k]);
    return s;
}

/* src/anuga_cuda/update_centroids_of_velocities_and_height/
 * update_centroids_of_velocities_and_height.cu:1-52 (boundary part): depth,
 * velocities at the boundary slots from the boundary values. */
void swcpu_boundary_velocities_and_height(const swcpu_domain *D, double *h, double *u,
                                          double *v)
{
    const double H0 = 1.0e-8;
    long m;
    for (m = 0; m < D->number_of_boundary_elements; m++) {
        double hm = D->stage_boundary_values[m] - D->bed_boundary_values[m], f;
        if (hm < 0)
            hm = 0;
        f = hm / (hm * hm + H0);
        h[m] = hm;
        u[m] = D->xmom_boundary_values[m] * f;
        v[m] = D->ymom_boundary_values[m] * f;
    }
}

/* src/anuga_cuda/update_centroids_of_velocities_and_height/
 * update_centroids_of_velocities_and_height.cu:1-52 (centroid part). */
void swcpu_velocities_and_height(const swcpu_domain *D, double *h, double *u,
                                 double *v)
{
    const double H0 = 1.0e-8;
    long k;
    for (k = 0; k < D->number_of_elements; k++) {
        double hk = D->stage_centroid_values[k] - D->bed_centroid_values[k], f;
        if (hk < 0)
            hk = 0;
        f = hk / (hk * hk + H0);
        h[k] = hk;
        u[k] = D->xmom_centroid_values[k] * f;
        v[k] = D->ymom_centroid_values[k] * f;
    }
}
