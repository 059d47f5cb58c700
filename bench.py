#!/usr/bin/env python
"""bench.py -- triangle-steps/s of ANUGA's explicit shallow-water evolve step
on one GB300, printed as one JSON line.

Workload: the 4,000,000-triangle wet/dry case (1000 x 1000 rectangular_cross
cells on 10 km x 10 km, 1:100 beach + Gaussian bumps, 2 m hump, per-triangle
Manning n), seeded synthetic data.  A step is one Euler step of the whole
mesh: fluxes + gravity, timestep reduction, friction + update + protect,
extrapolation + balance + boundaries.

  value       mixed-precision path, device time of K steps (CUDA events on
              the library's stream), inputs resident in HBM; the state is
              ~1.1 GB so every step streams from HBM (no L2 flush needed)
  e2e         the same K steps through the public C ABI from host buffers:
              H2D of the initial conserved state from pinned memory, evolve
              start, K steps, D2H of the final conserved state, host clock
  fp64        the FP64 parity path on the same K steps, with its FP64-pipe
              roofline (it is bound by GB300's FP64 rate, not HBM)
  mixed_error fresh 1,000-step runs in both precisions: per conserved
              quantity the max and RMS difference (normwise), and the depth
              of wet triangles per element
  roofline    the dominant kernel's algorithmic bytes per launch / its mean
              CUDA-event duration, against MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the CPU oracle (serial C restatement of the reference's
              ANUGA C path) on a bounded sample of the same workload; the
              oracle's final state is compared with the FP64 GPU path after
              the same steps (fp64_vs_oracle)
  configs     the 40,000-triangle dam break to t = 5 s and the 45,000-triangle
              tidal harbour for 2,000 steps: FP64 and mixed triangle-steps/s
              over the whole run, the oracle on one core beside them
  autotune    the tuned launch shape against a fixed 256-thread shape
  ensemble    the batched ensemble (256 inflow harbours by default) in runs/s,
              with the oracle on all host cores as its CPU baseline

--impl reference times the oracle on the host cores (one process per core,
each evolving the full workload for a bounded time) and prints the same line
with "impl": "reference".

Multi-GPU (torchrun): replicas only -- every rank evolves its own copy of the
workload; value = total triangle-steps of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "anuga-cuda_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "triangle-steps/s on 1 GB300 (mixed precision; FP64 alongside)"
UNIT = "triangle-steps/s"

# algorithmic bytes per triangle-step of each kernel (own arrays, neighbour
# gathers counted as cache hits)
MIXED_BYTES = {"flux": 128, "update": 104, "distribute": 114}
# DRAM bytes (read + write) per launch from one ncu capture of the 4,000,000-
# triangle mesh (1000x1000 cells); scaled by the triangles for other meshes
NCU_TRAFFIC_4M = {"flux": 509.35e6, "update": 377.39e6, "distribute": 520.23e6}
FP64_BYTES = {"flux": 296, "update": 120, "distribute": 253}
MODEL_BYTES = {"mixed": 368, "fp64": 568}   # whole-step byte model
ACC_STEPS = 1000                             # steps of the mixed-vs-FP64 accuracy check
WET_FLOOR = 0.01                             # m: wet triangles of the per-element depth error
# FP64-pipe thread instructions per triangle of each FP64 kernel (ncu
# sm__thread_inst_executed_pipe_fp64_pred_on.sum / triangles, 1,000,000-
# triangle wet/dry mesh after 48 steps) and the FP64 pipe's rate: GB300 runs
# FP64 at 1/64 of the FP32 rate, 2 thread instructions per SM per clock
# (DADD, DMUL, DFMA and the pipe's other instructions one slot each):
# 152 SMs x 2 x 2.07 GHz
FP64_PIPE_INST = {"flux": 494.99, "update": 166.79, "distribute": 317.03}
FP64_PIPE_PEAK = 152 * 2 * 2.07e9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=16)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cells", type=int, default=1000, help="rectangular_cross cells per side")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--ensemble", type=int, default=256,
                    help="scenarios of the batched-ensemble measurement (0: skip)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the dam-break and harbour measurements")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--ensemble-finaltime", type=float, default=3600.0)
    ap.add_argument("--surrogate", action="store_true",
                    help="also measure the BF16 MLP surrogate (trains on solver runs)")
    ap.add_argument("--surrogate-cells", type=int, default=224)
    ap.add_argument("--surrogate-train", type=int, default=2048)
    ap.add_argument("--surrogate-test", type=int, default=512)
    ap.add_argument("--surrogate-cal", type=int, default=256)
    ap.add_argument("--surrogate-steps", type=int, default=20000)
    ap.add_argument("--surrogate-only", action="store_true",
                    help="measure only the surrogate workflow (one JSON line of its own)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower() in ("active", "1")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        return None


def build_workload(cells):
    from anuga_cuda import scenarios
    return scenarios.wet_dry(m=cells)


def run_ours(args, rank, world, local, sc):
    import ctypes as C
    import numpy as np
    import anuga_cuda
    from anuga_cuda import DEFAULT, GPU_domain, _lib
    from anuga_cuda._lib import check, f64p, lib

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    if rank == 0:
        anuga_cuda.build()
    if dist is not None:
        dist.barrier()
    L = lib()
    if world > 1:
        # the library works on the current device of the calling thread
        cudart = C.CDLL("libcudart.so")
        cudart.cudaSetDevice(local)

    N = sc.N
    K, W = args.steps, args.warmup
    results = {}
    for prec in ("mixed", "fp64"):
        d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision=prec)
        sc.apply_to(d)
        d.evolve_steps(W)                      # warm-up; builds the step graph
        st = _lib.State_t()
        ms = C.c_double()
        if dist is not None:
            dist.barrier()
        with ClockSampler(local) as clk:
            check(L.swgpu_evolve_run_timed(d._h, K, C.byref(st), C.byref(ms)), d._h)
        if dist is not None:
            t = torch.tensor([ms.value], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_max = float(t.item())
        else:
            ms_max = ms.value
        assert st.total_steps == W + K, (st.total_steps, W + K)
        kms = (C.c_double * 4)()
        kp = min(K, 32)
        check(L.swgpu_profile_steps(d._h, kp, kms), d._h)
        results[prec] = {"ms": ms_max, "clocks": clk.summary(),
                         "kernel_ms": [kms[i] / kp for i in range(4)], "time": st.time}
        del d

    # accuracy: fresh runs of exactly ACC_STEPS steps in both precisions
    finals = {}
    for prec in ("mixed", "fp64"):
        d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision=prec)
        sc.apply_to(d)
        d.evolve_steps(ACC_STEPS)
        finals[prec] = {q: d.quantities[q].centroid_values
                        for q in ("stage", "xmomentum", "ymomentum", "elevation")}
        del d
    mixed_error = mixed_vs_fp64(finals["mixed"], finals["fp64"])

    # end to end through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        import torch
        host = {q: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
                for q, a in (("w", sc.stage_centroid), ("u", sc.xmom_centroid),
                             ("v", sc.ymom_centroid))}
        outs = {q: torch.empty(N, dtype=torch.float64).pin_memory() for q in ("w", "u", "v")}
        d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision="mixed")
        sc.apply_to(d)
        d.evolve_steps(W)

        def ptr(t):
            return C.cast(t.data_ptr(), _lib._f64p)

        st = _lib.State_t()

        def through_the_abi(steps):
            for qid, q in ((_lib.STAGE, "w"), (_lib.XMOMENTUM, "u"), (_lib.YMOMENTUM, "v")):
                check(L.swgpu_set_quantity(d._h, qid, ptr(host[q]), None, None), d._h)
            check(L.swgpu_evolve_start(d._h, 0.0, 1.0e300, -1.0), d._h)
            check(L.swgpu_evolve_run(d._h, steps, C.byref(st)), d._h)
            for qid, q in ((_lib.STAGE, "w"), (_lib.XMOMENTUM, "u"), (_lib.YMOMENTUM, "v")):
                check(L.swgpu_get_quantity(d._h, qid, ptr(outs[q]), None, None), d._h)

        # warm-up pass of W steps through the same calls and buffers (the
        # first transfers from freshly pinned host pages cost ~9 ms each)
        through_the_abi(W)
        check(L.swgpu_synchronize(d._h), d._h)
        t0 = time.perf_counter()
        through_the_abi(K)
        t1 = time.perf_counter()
        assert st.total_steps == K
        e2e = {"value": N * K / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": 3 * 8 * N / K, "d2h_bytes_per_step": 3 * 8 * N / K,
               "wall_s": t1 - t0}
        del d

    if dist is not None:
        dist.barrier()
    out = {"results": results, "mixed_error": mixed_error, "e2e": e2e, "N": N}
    out["dist"] = dist
    return out


def mixed_vs_fp64(m, f):
    """Per conserved quantity: max and RMS of |mixed - FP64| relative to the
    FP64 field's max and RMS (normwise); and over wet triangles (FP64 depth
    above WET_FLOOR) the largest |h_mixed - h_fp64| / h_fp64."""
    import numpy as np
    out = {"steps": ACC_STEPS, "against": "the FP64 GPU path (pinned to the oracle)"}
    for q in ("stage", "xmomentum", "ymomentum"):
        d = np.abs(m[q] - f[q])
        out[q] = {"max_rel": float(d.max() / np.abs(f[q]).max()),
                  "rms_rel": float(np.sqrt(np.mean(d ** 2)) / np.sqrt(np.mean(f[q] ** 2)))}
    z = f["elevation"]
    h64, hm = f["stage"] - z, m["stage"] - z
    wet = h64 > WET_FLOOR
    out["wet_depth_max_rel"] = float(np.max(np.abs(hm[wet] - h64[wet]) / h64[wet]))
    out["wet_floor_m"] = WET_FLOOR
    out["definition"] = ("max|q_mixed - q_fp64| / max|q_fp64| over triangles (rms likewise); "
                         "wet depth: max over triangles with h_fp64 > wet_floor_m of "
                         "|h_mixed - h_fp64| / h_fp64")
    return out


def host_cpu():
    """The host CPU's model name and core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not name:
        import platform
        name = platform.processor() or platform.machine()
    return {"model": name, "cores": os.cpu_count()}


def timed_run(d, steps=None, finaltime=None):
    """Device time (CUDA events on the library's stream) of one evolve from
    the domain's current state: ``steps`` steps, or to ``finaltime``; after
    an untimed run of the same length has built the step graph."""
    import ctypes as C
    from anuga_cuda import _lib
    from anuga_cuda._lib import check, lib
    L = lib()
    st, ms = _lib.State_t(), C.c_double()
    check(L.swgpu_evolve_start(d._h, 0.0, 1.0e300, -1.0 if finaltime is None else finaltime),
          d._h)
    check(L.swgpu_evolve_run_timed(d._h, 0 if steps is None else steps, C.byref(st),
                                   C.byref(ms)), d._h)
    return ms.value, st


def run_config(sc, steps=None, finaltime=None, cpu_seconds=3.0):
    """FP64 and mixed triangle-steps/s of a whole run of scenario ``sc`` (the
    same run twice per precision, the second timed), and the oracle's rate on
    one core over a bounded sample of the same run."""
    from anuga_cuda import DEFAULT, GPU_domain
    out = {"workload": sc.name, "triangles": sc.N}
    for prec in ("fp64", "mixed"):
        d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision=prec)
        sc.apply_to(d)
        timed_run(d, steps, finaltime)
        sc.apply_to(d)
        ms, st = timed_run(d, steps, finaltime)
        out[prec] = {"value": sc.N * st.total_steps / (ms / 1000.0), "unit": UNIT,
                     "steps": int(st.total_steps), "model_time_s": st.time,
                     "ms_per_step": ms / st.total_steps}
        del d
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    rate, n, wall, _ = cpu_oracle_rate(sc, seconds=cpu_seconds)
    out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": f"{n} steps ({wall:.1f} s) of the same run on one core"}
    out["mixed_over_cpu"] = out["mixed"]["value"] / rate
    return out


def run_autotune(sc, steps):
    """The autotuner's shape against the fixed 256-thread shape (every
    kernel 256 threads / triangles per tile, 16 steps per graph): device
    time of ``steps`` mixed steps from the initial state with each."""
    from anuga_cuda import DEFAULT, GPU_domain, autotune
    d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision="mixed")
    sc.apply_to(d)
    d.evolve_steps(0)
    rec = autotune.tune_handle(d._h, steps=32)
    shapes = {"fixed_256": {"flux_block": 256, "update_block": 256, "distribute_block": 256,
                            "steps_per_graph": 16, "flux_pipelined": 0},
              "tuned": rec["config"]}
    out = {"workload": sc.name, "triangles": sc.N, "steps": steps, "tuned_config": rec["config"]}
    for name, cfg in shapes.items():
        autotune.set_config(d._h, cfg)
        sc.apply_to(d)
        timed_run(d, steps)
        sc.apply_to(d)
        ms, st = timed_run(d, steps)
        out[name + "_ms_per_step"] = ms / st.total_steps
    out["speedup"] = out["fixed_256_ms_per_step"] / out["tuned_ms_per_step"]
    del d
    return out


def reduce_over_ranks(values, dist, op="max"):
    """Element-wise max (or sum) of a list of floats over all ranks (any
    backend; identity without torch.distributed)."""
    if dist is None:
        return list(values)
    import torch
    t = torch.tensor(values, dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return [float(v) for v in t.cpu()]


def run_ensemble(count, finaltime, rank=0, world=1, dist=None):
    """Batched ensemble of inflow harbours (N log-uniform in [5k, 200k],
    hydrograph peak U[50, 500] m^3/s, rise U[300, 1800] s, Manning n
    U[0.01, 0.05]; seed 4), mixed precision, every scenario from rest to
    ``finaltime``; device time of the whole run (CUDA events around the
    graph launches).  With several ranks the scenarios are sharded (no
    exchange) and the time is the slowest rank's."""
    import numpy as np
    from anuga_cuda import DEFAULT, scenarios
    from anuga_cuda.ensemble import Ensemble, shard
    specs = scenarios.ensemble_harbour_specs(count, seed=4)
    mine = shard([sp[2] ** 1.5 for sp in specs], rank, world)
    t0 = time.perf_counter()
    scs = scenarios.ensemble_harbours(count, seed=4, processes=os.cpu_count() or 1, only=mine)
    gen_s = time.perf_counter() - t0
    ens = Ensemble(scs, DEFAULT, "mixed")
    ms = ens.run_timed(finaltime)
    st = ens.states()
    steps = np.array([s.total_steps for s in st], dtype=np.float64)
    n = np.array([sc.N for sc in scs], dtype=np.float64)
    done_local = sum(1 for s in st if s.status == 0 and abs(s.time - finaltime) <= 1e-9 * finaltime)
    ms, = reduce_over_ranks([ms], dist, "max")
    done, work, ntot = reduce_over_ranks([done_local, float((n * steps).sum()), float(n.sum())],
                                         dist, "sum")
    smin, = reduce_over_ranks([-float(steps.min())], dist, "max")
    smax, = reduce_over_ranks([float(steps.max())], dist, "max")
    return {"metric": "ensemble runs/s", "value": done / (ms / 1000.0), "unit": "runs/s",
            "higher_is_better": True, "scenarios": count, "completed": int(done),
            "finaltime_s": finaltime, "wall_s": ms / 1000.0, "precision": "mixed",
            "ranks": world, "scaling": "strong (scenarios sharded across ranks)",
            "triangles_total": int(ntot), "steps_min": int(-smin),
            "steps_max": int(smax),
            "triangle_steps_per_s": work / (ms / 1000.0),
            "work_per_run": work / max(done, 1.0),
            "generation_s": gen_s,
            "workload": f"{count} inflow harbours (2 km x 1 km, Delaunay of seeded Poisson-disk "
                        "points, GRF bed), N log-uniform [5k, 200k], triangular hydrograph "
                        "peak U[50,500] m3/s rise U[300,1800] s, n U[0.01,0.05], seed 4"}


def run_surrogate(args):
    """The learned surrogate on its family mesh (the wet/dry generator at
    224 x 224 cells: 200,704 triangles): solver runs (batched ensembles,
    mixed precision, per-triangle tracking) for the training, calibration
    and held-out parameter sets (seeds 5000, 7000, 9000); BF16 training of
    the 16 -> 256 -> 256 -> 256 -> 3 network on the tcgen05 tensor cores;
    calibration of its error estimate; inference on the held-out set; and
    the answer within 5 cm (band re-solves of the flagged blocks) timed
    against the solver alone on the same scenarios (device time)."""
    import numpy as np
    from anuga_cuda import surrogate as SG
    t0 = time.perf_counter()
    fm = SG.FamilyMesh(cells=args.surrogate_cells)
    th_train = SG.sample_params(args.surrogate_train, seed=5000)
    th_cal = SG.sample_params(args.surrogate_cal, seed=7000)
    th_test = SG.sample_params(args.surrogate_test, seed=9000)
    hm, ta, ms_train = SG.solve(fm, th_train, batch=32)
    hmc, _, _ = SG.solve(fm, th_cal, batch=32)
    hmt, _, ms_test = SG.solve(fm, th_test, batch=32)
    solve_wall = time.perf_counter() - t0
    sg = SG.Surrogate(fm, seed=1)
    fit = sg.fit(th_train, SG.targets_from(fm, th_train, hm, ta),
                 steps=args.surrogate_steps, batch=32768, lr=1e-3)
    dc, _, ec, _ = sg.predict(th_cal)
    k, cal = SG.calibrate(ec, np.abs(dc - hmc), tol=0.05)
    sg.predict(th_test)                       # warm-up
    depth, _, err, infer_ms = sg.predict(th_test)
    rep = SG.evaluate(fm, th_test, hmt, ms_test, depth, err, infer_ms, k, tol=0.05)
    return {"mesh_triangles": fm.N, "train_scenarios": len(th_train),
            "calibration_scenarios": len(th_cal), "test_scenarios": len(th_test),
            "finaltime_s": SG.FINALTIME, "network": "16-256-256-256-3, BF16, tcgen05",
            "solver_ms_per_scenario": ms_test / len(th_test),
            "train_samples_per_s": fit["samples_per_s"], "train_tflops": fit["tflops"],
            "train_steps": fit["steps"], "train_batch": fit["batch"], "train_loss": fit["loss"],
            "inference_scenarios_per_s": len(th_test) / (infer_ms / 1000.0),
            "inference_rows_per_s": len(th_test) * fm.N / (infer_ms / 1000.0),
            "error_estimate_scale": k, "calibration": cal,
            "baseline_mae_m": float(np.abs(hmt - hm.mean(axis=0)[None]).mean()),
            "solver_wall_s": solve_wall, **rep}


def cpu_oracle_rate(sc, seconds=12.0, warm_steps=1):
    """Serial CPU oracle on the same workload for a bounded time: returns
    (triangle-steps/s, timed steps, wall seconds, the oracle domain after
    warm_steps + timed steps from the initial state)."""
    from anuga_cuda import DEFAULT
    from oracle import oracle as O
    O.build(ref=False)
    od = O.OracleDomain(sc.mesh, DEFAULT, sc.oracle_tags())
    sc.apply_to_oracle(od)
    od.evolve_start(1.0e300)
    od.evolve_steps(1.0e300, None, warm_steps)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        od.evolve_steps(1.0e300, None, 1)
        steps += 1
    wall = time.perf_counter() - t0
    return sc.N * steps / wall, steps, wall, od


def fp64_vs_oracle(sc, od, steps):
    """The FP64 GPU path after the oracle's ``steps`` steps from the same
    initial state: per conserved quantity max|gpu - oracle| / max|oracle|,
    and the water volumes' relative difference."""
    import numpy as np
    from anuga_cuda import DEFAULT, GPU_domain
    d = GPU_domain(mesh=sc.mesh, parameters=DEFAULT, precision="fp64")
    sc.apply_to(d)
    st = d.evolve_steps(steps)
    out = {"steps": int(st.total_steps), "model_time_equal": st.time == od.D.time}
    for q, pre in (("stage", "stage"), ("xmomentum", "xmom"), ("ymomentum", "ymom")):
        o = od.arrays[pre + "_centroid_values"]
        out[q + "_max_rel"] = float(np.max(np.abs(d.quantities[q].centroid_values - o)) /
                                    max(np.max(np.abs(o)), 1e-300))
    out["volume_rel"] = abs(d.get_water_volume() - od.mass()) / abs(od.mass())
    del d
    return out


def _ref_worker(args):
    cells, seconds, q = args
    sc = build_workload(cells)
    rate, steps, wall, _ = cpu_oracle_rate(sc, seconds)
    q.put((rate, steps, wall))


def _collect(q, ps, timeout):
    """One result per worker process from queue q, waiting at most
    ``timeout`` seconds in all; workers that have not answered by then (or
    died) are terminated and left out."""
    import queue as _queue
    res, end = [], time.perf_counter() + timeout
    while len(res) < len(ps):
        try:
            res.append(q.get(timeout=max(end - time.perf_counter(), 0.1)))
        except _queue.Empty:
            break
    for p in ps:
        p.join(timeout=max(end - time.perf_counter(), 1.0))
        if p.is_alive():
            p.terminate()
    if not res:
        raise RuntimeError("no CPU worker returned a result")
    return res


def _ensemble_cpu_worker(args):
    spec, seconds, q = args
    from anuga_cuda import scenarios
    sc = scenarios._inflow_harbour_args(spec)
    rate, steps, wall, _ = cpu_oracle_rate(sc, seconds)
    q.put((rate, steps, wall, sc.N))


def ensemble_cpu_baseline(specs, work_per_run, seconds=15.0):
    """The oracle on all host cores, one scenario of the ensemble per core
    (chosen evenly across the size range) for a bounded time each: the
    aggregate triangle-steps/s, and the runs/s it gives at the work per run
    (triangle-steps to the final time) the GPU run measured."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    order = sorted(range(len(specs)), key=lambda i: specs[i][2])
    pick = [order[int(round(j * (len(order) - 1) / max(cores - 1, 1)))]
            for j in range(min(cores, len(order)))]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_ensemble_cpu_worker, args=((specs[i], seconds, q),))
          for i in pick]
    for p in ps:
        p.start()
    res = _collect(q, ps, seconds + 600.0)
    total = sum(r[0] for r in res)
    return {"value": total / work_per_run, "unit": "runs/s", "cores": len(ps), "kind": "port",
            "triangle_steps_per_s": total,
            "sample": f"{len(ps)} processes, one scenario each ({min(r[3] for r in res)}-"
                      f"{max(r[3] for r in res)} triangles), ~{seconds:.0f} s of FP64 Euler "
                      f"steps; runs/s = aggregate triangle-steps/s / the "
                      f"{work_per_run:.3g} triangle-steps per run of the GPU ensemble"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    try:
        avail = int([l for l in open("/proc/meminfo") if l.startswith("MemAvailable")][0]
                    .split()[1]) * 1024
    except (OSError, IndexError):
        avail = 64 << 30
    per = 6.0e9 * (args.cells / 1000.0) ** 2     # oracle + mesh bytes per process
    procs = max(1, min(cores, int(0.6 * avail / per), 32))
    seconds = 30.0
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_ref_worker, args=((args.cells, seconds, q),)) for _ in range(procs)]
    t0 = time.perf_counter()
    for p in ps:
        p.start()
    res = _collect(q, ps, seconds + 600.0)
    procs = len(res)
    wall = time.perf_counter() - t0
    total = sum(r[0] for r in res)
    steps = sum(r[1] for r in res)
    N = 4 * args.cells * args.cells
    line = {
        "impl": "reference", "metric": METRIC, "value": total, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * N / total,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded wet/dry scenario)",
        "config": {"workload": f"wet_dry {args.cells}x{args.cells} rectangular_cross "
                               f"({N} triangles)", "triangles": N},
        "cpu_baseline": {"value": total, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{procs} processes x ~{seconds:.0f} s of full-mesh Euler "
                                   f"steps ({steps} steps in total, {wall:.0f} s wall)"},
        "e2e": {"value": total, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line))
        return
    if args.surrogate_only:
        if rank == 0:
            print(json.dumps({"metric": "surrogate time to answer within 5 cm vs solver alone",
                              "surrogate": run_surrogate(args)}))
        return
    sc = build_workload(args.cells)
    out = run_ours(args, rank, world, local, sc)
    dist = out.pop("dist")
    ens = None
    if args.ensemble > 0:  # every rank runs its shard of the scenarios
        ens = run_ensemble(args.ensemble, args.ensemble_finaltime, rank, world, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    N, K, W = out["N"], args.steps, args.warmup
    r = out["results"]
    mixed_ms, fp64_ms = r["mixed"]["ms"], r["fp64"]["ms"]
    value = world * N * K / (mixed_ms / 1000.0)
    fp64_value = world * N * K / (fp64_ms / 1000.0)
    peaks = measured_peaks()
    peak_gbs = peaks["hbm_gbs"] if peaks else 6800.0
    kms = r["mixed"]["kernel_ms"]
    names = ["flux", "update", "distribute"]
    dom = max(range(3), key=lambda i: kms[i])
    achieved = MIXED_BYTES[names[dom]] * N / (kms[dom] / 1000.0) / 1e9
    kms64 = r["fp64"]["kernel_ms"]
    fp64_pipe = {}
    for i, k in enumerate(names):
        if FP64_PIPE_INST[k]:
            a = FP64_PIPE_INST[k] * N / (kms64[i] / 1000.0)
            fp64_pipe[k] = {"achieved": a, "frac": a / FP64_PIPE_PEAK}
    if fp64_pipe:
        fp64_pipe.update({"unit": "FP64-pipe thread instructions/s", "peak": FP64_PIPE_PEAK,
                          "peak_source": "152 SMs x 2 FP64 lanes per SM per clock x 2.07 GHz",
                          "instructions_source": "ncu sm__thread_inst_executed_pipe_fp64_pred_on"
                                                 ".sum per triangle, 1,000,000-triangle mesh"})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": mixed_ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64 mixed", "data": "synthetic (seeded wet/dry scenario)",
        "config": {"workload": f"wet_dry {args.cells}x{args.cells} rectangular_cross ({N} triangles)",
                   "triangles": N, "precision": "mixed", "l2": "inputs larger than L2 (state ~1.1 GB)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": fp64_ms / K,
                 "kernel_ms": dict(zip(names, kms64)),
                 "mixed_over_fp64": value / fp64_value,
                 "hbm_frac": MODEL_BYTES["fp64"] * N / (fp64_ms / K / 1000.0) / 1e9 / peak_gbs,
                 "fp64_pipe_roofline": fp64_pipe or None},
        "mixed_error": out["mixed_error"],
        "kernel_ms": dict(zip(names + ["step_clock"], kms)),
        "roofline": {"bound": "hbm", "kernel": names[dom] + "_mixed", "achieved": achieved,
                     "peak": peak_gbs, "unit": "GB/s", "frac": achieved / peak_gbs,
                     "traffic": NCU_TRAFFIC_4M[names[dom]] * N / 4.0e6,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                       "capture of the 4,000,000-triangle mesh"
                                       + ("" if N == 4000000 else ", scaled to this mesh"),
                     "peak_source": "measured" if peaks else "fallback",
                     "step_model_frac": MODEL_BYTES["mixed"] * N / (mixed_ms / K / 1000.0) / 1e9
                     / peak_gbs},
        "clocks": r["mixed"]["clocks"],
        # the timed region issues K steps of 4 kernels (flux, step clock,
        # update, distribute): whole graphs of 16 steps, then the remainder
        "gpu_launches": 4 * K,
        "host_cpu": host_cpu(),
    }
    if out["e2e"]:
        line["e2e"] = {k: out["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step",
                                                     "d2h_bytes_per_step")}
    if not args.no_cpu_baseline:
        rate, steps, wall, od = cpu_oracle_rate(sc, seconds=12.0)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "cpu": host_cpu()["model"],
                                "sample": f"{steps} Euler steps of the full {N}-triangle mesh "
                                          f"({wall:.1f} s) on one core"}
        line["fp64_vs_oracle"] = fp64_vs_oracle(sc, od, steps + 1)
        del od
    if not args.no_configs:
        from anuga_cuda import scenarios
        line["configs"] = {
            "dam_break_40k": run_config(scenarios.dam_break(), finaltime=5.0),
            "tidal_harbour_45k": run_config(scenarios.tidal_harbour(), steps=2000)}
    if not args.no_autotune:
        from anuga_cuda import scenarios
        line["autotune"] = {"tidal_harbour_45k": run_autotune(scenarios.tidal_harbour(), 400),
                            "wet_dry_4M": run_autotune(sc, 64)}
    if ens is not None:
        if not args.no_cpu_baseline:
            from anuga_cuda import scenarios
            ens["cpu_baseline"] = ensemble_cpu_baseline(
                scenarios.ensemble_harbour_specs(args.ensemble, seed=4), ens["work_per_run"])
        line["ensemble"] = ens
    if args.surrogate:
        line["surrogate"] = run_surrogate(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
