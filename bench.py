"""Benchmark of the level-set transport step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload fwdadj|batched|fp64|sussman|hybrid|adjcheck]

Default workload ("fwdadj"): the large free-surface case, 512 x 256 x 256
curvilinear nodes (x = 16 xi + 0.05 sin(2 pi eta), y = 4 eta, z = 2 zeta^1.3),
phi0 = z - 1 - 0.08 sech^2(k(x-4)) (1 + 0.2 cos(2 pi y / 4)), solitary-wave
velocity, CFL 0.4, 10 reinitialisation pseudo-steps per step, FP64 water
volume and mass correction (towards the initial volume) every step.  One
benchmark step = the whole 200-step run of the FP32 batched path (autotuned
tile shape) from phi0 with a checkpoint every 20 steps, followed by the
hand-written adjoint's reverse sweep, seeded with dL/dphi_T of a linear loss
with seeded weights: the sweep reverses the last segment from the internals
the forward kept and recomputes each of the 9 earlier segments from its
checkpoint before reversing it.  Beside it: the plain FP64 GPU path
(lsm_levelsetmethod, the reference's arithmetic) on the same grid, timed;
and the narrow-band phi error and volume drift of the FP32 run after 200
steps against the same 200 steps in FP64 (the batch's FP64 instantiation,
which matches the FP64 oracle to 1e-12, with the same mass correction).

"batched" workload: 64 independent instances with per-axis sizes drawn from
{32..96} (numpy seed 0), identity-plus-random-shear grids, Fourier phi0,
divergence-free curl velocity, CFL 0.5, 5 reinitialisation pseudo-steps per
step, forward only.

"fp64" workload: the curvilinear solitary-wave case, 256 x 128 x 96 nodes,
10 reinitialisation pseudo-steps per step, through `lsm_levelsetmethod` in
the reference's FP64 arithmetic.  "sussman": the same with the
reference's live reinitialisation (`reinitialisation_test2`, reinit_scheme 1).
"hybrid": the same with the reference deck's hybrid branch (advection of the
AdvectionNodes band, geometric reinitialisation).

Metric: Gcell-steps/s = grid nodes x physical steps / second (whole job;
for "fwdadj" each cell-step is forward + adjoint).
  value : device-resident inputs, CUDA events on the launching stream.
  e2e   : the same through the C-ABI with host arrays: phi0, q and the
          loss seed copied in, phi_T and both gradients copied out.
Synthetic inputs with the workloads' shapes and value distributions (the
reference ships no input decks).  The reference arm (--impl reference)
times the CPU FP64 restatement of the reference (the Fortran/MPI original
cannot be built: no Fortran compiler) with all host threads; the reference
has no adjoint, so its figure is forward only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "ns-lsm-single-phase_gb300"))

WORKLOAD = dict(ni=256, nj=128, nk=96, reinit_iters=10, redistance=50)

# algorithmic HBM words per node for one launch of each kernel (FP64 = 8 bytes)
ALGO_WORDS = {
    "rk_stage_kernel": 20.0 / 3.0,   # stages read phi_prev, phi^n (stages 2-3), U(3), aj; write phi
    "reinit_step_kernel": 15.0,      # d, s, phi0, |grad phi0|, delta, metrics(9); write d
    "sign_ini_kernel": 13.0,         # phi0, metrics(9); write s, |grad phi0|, delta
    "contra_kernel": 16.0,           # u,v,w, metrics(9), aj; write U(3)
    "volume_kernel": 4.0,            # phi, x, y, z
    "bc_full_kernel": 2.0,
    "copy_kernel": 2.0,
    "normgrad_d_kernel": 12.0,       # phi, phizero, metrics(9); |grad phi|
    "sussman_rk_kernel": 6.0,        # dn, dn1 (rmw), |grad|, |grad| at the iteration start, sign
    "minmax_partial_kernel": 1.0,
}


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def dist_setup(n_gpus):
    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(_env_int("LOCAL_RANK", 0))
    return rank, world


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

    def mark(self, t0, t1):
        """Keep the samples taken inside [t0, t1] (the timed region)."""
        self.window = (t0, t1)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = self.rows
        if self.window:
            inside = [r for r in rows if self.window[0] - 0.1 <= r[0] <= self.window[1] + 0.1]
            if inside:
                rows = inside
            elif rows:   # region shorter than the sampling period: the nearest sample
                mid = 0.5 * (self.window[0] + self.window[1])
                rows = [min(rows, key=lambda r: abs(r[0] - mid))]
        for _, r in rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workload
FP64_METRIC = {
    0: "Gcell-steps/s (plain FP64 level-set step: WENO3-RK3 advection + reinitialisation + volume)",
    1: "Gcell-steps/s (plain FP64 level-set step with the live Sussman reinitialisation: WENO3-RK3 advection + "
       "reinitialisation_test2 + volume)",
    2: "Gcell-steps/s (plain FP64 level-set step, hybrid branch: WENO3-RK3 advection of the AdvectionNodes band + "
       "geometric reinitialisation + volume)",
}
FP64_REINIT = {0: "reinitialization", 1: "reinitialisation_test2, ENO2 gradients, TVD-RK3 pseudo time",
               2: "geometric_reinitialisation: marching-tetrahedra isosurface, distances of the nodes within 4 of it"}
FP64_SCHEME = {"fp64": 0, "sussman": 1, "hybrid": 2}


def make_case(ni, nj, nk, reinit_iters, scheme=0):
    """scheme 0: `reinitialization`; 1: the reference's live `reinitialisation_test2`;
    2: the hybrid branch (geometric reinitialisation, the reference deck's setting)"""
    from nslsm import configs
    case = configs.solitary_wave(ni, nj, nk, reinit_iters=reinit_iters)
    if scheme == 2:
        case.params = case.params.replace(hybrid_reinitialisation=True)
    else:
        case.params = case.params.replace(reinit_scheme=scheme)
    return case


def prepare_device(case, ls, torch):
    """Upload inputs, compute metrics on the GPU, redistance phi0, set dt."""
    from nslsm import LsmParams  # noqa: F401
    g = case.grid

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()

    x, y, z = dev(case.x), dev(case.y), dev(case.z)
    csi, eta, zet, aj = ls.mg_metrics(g, x, y, z)
    q = dev(case.q(0.0))
    # CFL time step in computational space (csi/eta/zet . u)
    u = q[..., 1:4]
    smax = max(float((m * u).sum(-1).abs().max()) for m in (csi, eta, zet))
    p = case.params.replace(delti_lsm=case.cfl / smax)
    phi = dev(case.phi0)
    if case.redistance_iters:
        pr = p.replace(RNitermax=case.redistance_iters)
        phi = ls.reinitialization(g, pr, phi, csi, eta, zet)
        ls.bcond_lsm(g, pr, phi)
    return dict(g=g, p=p, q=q, csi=csi, eta=eta, zet=zet, aj=aj, phi=phi, x=x, y=y, z=z)


def roofline_from_profile(prof, n_nodes, peaks):
    if not prof:
        return None
    name, (launches, ms) = max(prof.items(), key=lambda kv: kv[1][1])
    words = ALGO_WORDS.get(name)
    avg_s = ms / 1e3 / max(launches, 1)
    achieved = None if words is None else words * 8.0 * n_nodes / avg_s / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0)) if peaks else 6800.0
    traffic = read_traffic(name, n_nodes)
    total = sum(v[1] for v in prof.values())
    if words is None and name.startswith("k_geo_"):
        # the geometric reinitialisation's distance loops: FP64 arithmetic on
        # irregular lists, no HBM roofline (the FP64 pipe is the limit)
        total = sum(v[1] for v in prof.values())
        return {"bound": "fp64", "kernel": name, "achieved": None, "peak": None, "unit": None, "frac": None,
                "traffic": None, "avg_launch_us": avg_s * 1e6, "share": ms / total if total else None,
                "note": "FP64-issue bound distance loops over the interface lists; see the ncu summary"}
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": None if achieved is None else achieved / peak, "traffic": traffic,
            "algorithmic_bytes_per_launch": None if words is None else words * 8.0 * n_nodes,
            "avg_launch_us": avg_s * 1e6, "share": ms / total if total else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s"}


def read_traffic(kernel, n_nodes):
    """DRAM bytes per launch from the committed ncu summary (bytes per node,
    measured on a smaller case and scaled by the node count)."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == "traffic" and parts[1] == kernel:
            try:
                return float(parts[2]) * n_nodes
            except ValueError:
                return None
    return None


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------- CPU baseline
def cpu_oracle_time(case, steps, threads, warmup=0):
    """Seconds per physical step of the CPU FP64 oracle (OpenMP build) on
    `case`, timed over `steps` steps after `warmup` untimed ones."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    O.build()
    orc = O.Oracle(omp=True)
    g = O.make_grid(case.grid.ni, case.grid.nj, case.grid.nk)
    csi, eta, zet, aj = orc.mg_metrics(g, case.x, case.y, case.z)
    q = case.q(0.0)
    u = q[1:4]
    smax = max(float(np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2]).max()) for m in (csi, eta, zet))
    cp = case.params
    p = O.make_params(epslsm=cp.epslsm, delti_lsm=case.cfl / smax, RNitermax=cp.RNitermax,
                      RNtimestep=cp.RNtimestep, isnarrow=cp.isnarrow, narrowcoef=cp.narrowcoef,
                      reinit_scheme=cp.reinit_scheme, epsReinitialisation=cp.epsReinitialisation,
                      hybrid_reinitialisation=int(cp.hybrid_reinitialisation),
                      OrderReinitialisationBoundaries=cp.OrderReinitialisationBoundaries,
                      ENOBCReinitialisation=int(cp.ENOBCReinitialisation))
    phi = case.phi0
    for it in range(1, warmup + 1):
        phi, _ = orc.levelsetmethod(g, p, q, csi, eta, zet, aj, phi, phi, case.x, case.y, case.z, it)
    t0 = time.perf_counter()
    for it in range(warmup + 1, warmup + steps + 1):
        phi, _ = orc.levelsetmethod(g, p, q, csi, eta, zet, aj, phi, phi, case.x, case.y, case.z, it)
    return (time.perf_counter() - t0) / steps, orc.threads


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------- batched FP32 arm
BATCH = dict(n_inst=64, lo=32, hi=96, seed=0, reinit_iters=5, cfl=0.5)

# algorithmic HBM bytes per node for one launch of the batched FP32 kernels
BATCH_ALGO_BYTES = {
    "k_stage_z": 17.0 / 3.0 * 4,   # phi_prev, phi^n (stages 2-3), W(3); phi
    "k_reinit_z": 12.0 * 4,      # d, s, metrics(9); d
    "k_sign_reinit_z": 12.0 * 4, # phi0, metrics(9); s, d
    "k_reinit": 12.0 * 4,        # brick-table pseudo-step: d, s, metrics(9); d
    "k_sign_reinit": 12.0 * 4,   # brick-table first pseudo-step: phi0, metrics(9); s, d
    "k_contra": 15.0 * 4,        # u(3), metrics(9); W(3)
    "k_vol_scan_z": 4.0 + 8.0,   # phi (FP32) + fixed-point cell volume (interface cells listed for k_vol_iface)
    "k_bc_full": 8.0,
}


def batch_setup(torch, ls, stream, reinit_iters, use_graph=True, autotune=True, shape=0, n_inst=None):
    """Build the 64-instance workload on the GPU: FP64 metrics per instance
    (lsm_mg_metrics), CFL time step per instance, packed FP32 batch."""
    from nslsm import configs
    from nslsm.batch import LevelSetBatch
    kw = dict(BATCH)
    if n_inst:
        kw["n_inst"] = n_inst
    insts = configs.batched_instances(kw["n_inst"], kw["lo"], kw["hi"], kw["seed"], kw["cfl"])

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()

    meta = []
    for it in insts:
        csi, eta, zet, aj = ls.mg_metrics(it.grid, dev(it.x), dev(it.y), dev(it.z))
        u = dev(it.q)[..., 1:4]
        smax = max(float((m * u).sum(-1).abs().max()) for m in (csi, eta, zet))
        meta.append(dict(inst=it, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.cfl / smax))
    b = LevelSetBatch([(*m["inst"].grid.shape, m["dt"], m["inst"].dtau, m["inst"].eps) for m in meta],
                      RNitermax=reinit_iters, btype=(1,) * 6, BigPhi=5.0, stream=stream, use_graph=use_graph,
                      autotune=autotune, shape=shape)
    for k, m in enumerate(meta):
        it = m["inst"]
        b.set_geometry(k, dev(it.x), dev(it.y), dev(it.z), m["csi"], m["eta"], m["zet"])
        b.set_velocity(k, dev(it.q))
        b.set_phi(k, dev(it.phi0))
    return b, meta


def run_batched(args):
    import torch
    from nslsm import LevelSet, LsmParams
    from nslsm._lib import KernelTimer

    rank, world = dist_setup(args.gpus)
    dev_index = torch.cuda.current_device()
    R = BATCH["reinit_iters"]
    ls = LevelSet(device=dev_index)
    stream = torch.cuda.Stream()
    b, meta = batch_setup(torch, ls, stream.cuda_stream, R, n_inst=args.n_inst)
    n = b.nodes
    b.step(args.warmup, volumes=False)          # includes the tile autotune and graph capture
    torch.cuda.synchronize()
    dist_barrier(world)
    from nslsm import _lib
    lib = _lib.load()
    l0 = lib.lsm_kernel_launch_count(None)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev_index) as clocks:
        time.sleep(0.5)
        torch.cuda.synchronize()
        t_start = time.time()
        with torch.cuda.stream(stream):
            ev0.record(stream)
            b.step(args.steps, volumes=False)
            ev1.record(stream)
        torch.cuda.synchronize()
        clocks.mark(t_start, time.time())
        time.sleep(0.2)
    launches = lib.lsm_kernel_launch_count(None) - l0
    dist_barrier(world)
    ms = ev0.elapsed_time(ev1)
    ms_max = dist_max(ms, world)
    value = world * n * args.steps / (ms_max / 1e3) / 1e9
    shape = b.shape

    # per-kernel attribution: the same batch without the graph (the event
    # timer brackets each launch on the batch's stream)
    b2, _ = batch_setup(torch, ls, stream.cuda_stream, R, use_graph=False, autotune=False, shape=shape[0],
                        n_inst=args.n_inst)
    b2.step(2, volumes=False)
    torch.cuda.synchronize()
    with KernelTimer() as kt:
        b2.step(5, volumes=False)
        torch.cuda.synchronize()
        prof = kt.read()
    b2.close()
    roof = None
    if prof:
        name, (cnt, tms) = max(prof.items(), key=lambda kv: kv[1][1])
        byt = BATCH_ALGO_BYTES.get(name)
        avg = tms / 1e3 / max(cnt, 1)
        peaks = load_peaks()
        peak = float(peaks.get("hbm_gbs", 6800.0)) if peaks else 6800.0
        ach = None if byt is None else byt * n / avg / 1e9
        total = sum(v[1] for v in prof.values())
        roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": None if ach is None else ach / peak, "traffic": read_traffic(name, n),
                "algorithmic_bytes_per_launch": None if byt is None else byt * n, "avg_launch_us": avg * 1e6,
                "share": tms / total if total else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s",
                "per_kernel_frac": {k: (BATCH_ALGO_BYTES[k] * n / (v[1] / 1e3 / v[0]) / 1e9 / peak)
                                    for k, v in prof.items() if k in BATCH_ALGO_BYTES}}

    # the plain FP64 GPU path on the same instances (one levelsetmethod call per instance)
    fp64 = None
    if not args.no_fp64_compare:
        steps64 = 2
        tot64 = 0.0
        nodes64 = 0
        for m in meta[:16]:
            it = m["inst"]
            g = it.grid
            p = LsmParams(epslsm=it.eps, delti_lsm=m["dt"], RNitermax=R, RNtimestep=it.dtau, isnarrow=1,
                          narrowcoef=4.0, BigPhi=5.0)

            def dev(a):
                return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()
            q, x, y, z = dev(it.q), dev(it.x), dev(it.y), dev(it.z)
            phi = dev(it.phi0)
            phin = phi.clone()
            ls.set_stream(torch.cuda.current_stream().cuda_stream)
            ls.levelsetmethod(g, p, q, m["csi"], m["eta"], m["zet"], m["aj"], phi, phin, x, y, z, 1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for s in range(steps64):
                phin.copy_(phi)
                ls.levelsetmethod(g, p, q, m["csi"], m["eta"], m["zet"], m["aj"], phi, phin, x, y, z, s + 2)
            torch.cuda.synchronize()
            tot64 += time.perf_counter() - t0
            nodes64 += g.n * steps64
        v64 = nodes64 / tot64 / 1e9
        fp64 = {"value": v64, "unit": "Gcell-steps/s", "sample": "first 16 instances, %d steps each, "
                "lsm_levelsetmethod (reference FP64 arithmetic)" % steps64, "speedup_fp32_batched": value / v64}

    # end-to-end: every step copies each instance's velocity in from pinned
    # host memory and reads every instance's phi back
    pinned = []
    for m in meta:
        a = np.asfortranarray(m["inst"].q)
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        o = torch.empty(m["inst"].grid.n, dtype=torch.float64, pin_memory=True)
        pinned.append((v, t, o.numpy().reshape(m["inst"].grid.shape, order="F"), o))
    e2e_steps = max(2, min(args.steps, 5))
    qv, po = [p[0] for p in pinned], [p[2] for p in pinned]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        b.set_velocities(qv)          # every instance's q in one call (lsm_batch_set_velocities)
        b.step(1, volumes=True)
        b.get_phis(po)                # every instance's phi out in one call (lsm_batch_get_phis)
    torch.cuda.synchronize()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e_value = world * n * e2e_steps / e2e_s / 1e9

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = batch_cpu_baseline(meta[:6], R)
    if rank == 0:
        line = {
            "metric": "Gcell-steps/s (batched FP32 level-set step, forward: WENO3-RK3 + %d reinit pseudo-steps + "
                      "FP64 volume, 64 uneven instances)" % R,
            "value": value, "unit": "Gcell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (64 instances, sizes U{32..96} seed 0, shear metrics, Fourier phi0, "
                                    "curl velocity; the reference ships no decks)",
            "config": {"workload": "batched_instances 64 x U{32..96}^3 (%d nodes), CFL 0.5, %d reinit "
                                   "pseudo-steps/step, volume each step, one launch per pass, CUDA graph" % (n, R),
                       "nodes": n, "tile_shape": shape[1], "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (working set %.2f GB > 129 MB)" % (n * 4 * 30 / 1e9)},
            "roofline": roof,
            "cpu_baseline": cpu,
            "fp64_gpu_path": fp64,
            "e2e": {"value": e2e_value, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 8 * n + 32 * len(meta), "steps": e2e_steps},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
            "kernel_times_ms": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in prof.items()},
        }
        print(json.dumps(line))
    b.close()
    ls.close()


def batch_cpu_baseline(meta, R):
    """CPU FP64 oracle (OpenMP, all host threads) on a bounded sample of the
    batched workload: one physical step of each of the first instances."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    threads = host_threads()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    O.build()
    orc = O.Oracle(omp=True)
    nodes, sec = 0, 0.0
    for m in meta:
        it = m["inst"]
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = orc.mg_metrics(g, it.x, it.y, it.z)
        p = O.make_params(epslsm=it.eps, delti_lsm=m["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0)
        t0 = time.perf_counter()
        orc.levelsetmethod(g, p, it.q, csi, eta, zet, aj, it.phi0, it.phi0, it.x, it.y, it.z, 1)
        sec += time.perf_counter() - t0
        nodes += it.grid.n
    return {"value": nodes / sec / 1e9, "unit": "Gcell-steps/s", "cores": orc.threads, "kind": "port",
            "sample": "1 physical step of each of the first %d instances (%d nodes), CPU FP64 oracle, OpenMP"
                      % (len(meta), nodes)}


# ---------------------------------------------------------------- FP64 arm
def run_ours(args):
    if args.workload == "fwdadj":
        return run_fwdadj(args)
    if args.workload == "adjcheck":
        return run_adjcheck(args)
    if args.workload == "batched":
        return run_batched(args)
    return run_fp64(args)


# ------------------------------------------------- FP32 forward + adjoint arm
FWDADJ = dict(ni=512, nj=256, nk=256, reinit_iters=10, nsteps=200, ckpt=20, compare_steps=20)
FWDADJ_METRIC = ("Gcell-steps/s (batched FP32 level-set forward + adjoint: WENO3-RK3 + %d reinit pseudo-steps + "
                 "FP64 volume and mass correction; vs the plain FP64 GPU path)")
FWDADJ_WORKLOAD = ("large_free_surface %dx%dx%d curvilinear, CFL 0.4, %d RK3 steps, %d reinit pseudo-steps/step, "
                   "FP64 volume reduction and mass correction every step; adjoint with a checkpoint every %d steps "
                   "(one step = the whole run: forward from phi0, then the reverse sweep recomputing %d segments)")

# algorithmic HBM bytes per node for one launch of the FP32 batched kernels
# (each distinct array read once and written once; halos not counted)
FWDADJ_BYTES = {
    "k_contra": 15 * 4,            # u(3), metrics(9); W(3)
    "k_stage_z": 17.0 / 3.0 * 4,     # phi_prev, phi^n (stages 2-3), W(3); stage output
    "k_reinit_z": 12 * 4,          # d, s, metrics(9); d
    "k_sign_reinit_z": 12 * 4,     # phi0, metrics(9); s, d
    "k_reinit_rec_z": 18 * 4,      # d, s, metrics(9); d, adjoint coefficients(6)
    "k_sign_reinit_rec_z": 18 * 4, # phi0, metrics(9); s, d, adjoint coefficients(6)
    "k_adj_reinit_c": 8 * 4,       # lam, coefficients(6); lam_out
    "k_vol_scan_z": 4 + 8,         # phi (FP32) + fixed-point cell volume; interface cells listed
    "k_bc_full": 2 * 4,            # phi in, phi out
    "k_adj_stage_x": 8 * 4,        # in, W_x, lamP0, lamPhin (rmw), lamW_x (rmw); lam_in
    "k_adj_stage_y": 7 * 4,        # in, W_y, lamP0, lam_in (rmw), lamW_y (rmw)
    "k_adj_stage_z": 7 * 4,        # in, W_z, lamP0, lam_in (rmw), lamW_z (rmw)
    "k_adj_reinit": 13 * 4,        # d, s, metrics(9), lam; lam_out
    "k_adj_contra": 18 * 4,        # lamW(3), metrics(9), lam_u(3, rmw)
    "k_cvt_in": 8 + 4,
    "k_cvt_out": 4 + 8,
    "k_mass_shift": 2 * 4,         # phi in, phi out
    "k_tile_sum": 4,               # lam
    # k_vol_iface, k_mass_weights and k_mass_apply walk the interface-cell
    # list: their bytes scale with the interface, not with the node count
}


def _roofline(prof, n, peaks, table, dtype_note):
    name, (cnt, tms) = max(prof.items(), key=lambda kv: kv[1][1])
    byt = table.get(name)
    avg = tms / 1e3 / max(cnt, 1)
    peak = float(peaks.get("hbm_gbs", 6800.0)) if peaks else 6800.0
    ach = None if byt is None else byt * n / avg / 1e9
    total = sum(v[1] for v in prof.values())
    return {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": None if ach is None else ach / peak, "traffic": read_traffic(name, n),
            "algorithmic_bytes_per_launch": None if byt is None else byt * n, "avg_launch_us": avg * 1e6,
            "share": tms / total if total else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6800 GB/s",
            "bytes_note": dtype_note,
            "per_kernel_frac": {k: (table[k] * n / (v[1] / 1e3 / v[0]) / 1e9 / peak)
                                for k, v in prof.items() if k in table}}


def run_fwdadj(args):
    import torch
    from nslsm import LevelSet, LsmParams, configs, _lib
    from nslsm._lib import KernelTimer
    from nslsm.batch import LevelSetBatch

    rank, world = dist_setup(args.gpus)
    dev_index = torch.cuda.current_device()
    W = dict(FWDADJ)
    if args.grid:
        W["ni"], W["nj"], W["nk"] = (int(v) for v in args.grid.lower().split("x"))
    if args.segment:
        W["ckpt"] = args.segment
    if args.nsteps:
        W["nsteps"] = args.nsteps
    R, NS, CK = W["reinit_iters"], W["nsteps"], min(W["ckpt"], W["nsteps"])
    case = configs.large_free_surface(W["ni"], W["nj"], W["nk"], reinit_iters=R)
    g = case.grid
    n = g.n

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()

    ls = LevelSet(device=dev_index)
    stream = torch.cuda.Stream()
    x, y, z = dev(case.x), dev(case.y), dev(case.z)
    csi, eta, zet, aj = ls.mg_metrics(g, x, y, z)
    q = dev(case.q(0.0))
    phi0 = dev(case.phi0)
    smax = max(float((m * q[..., 1:4]).sum(-1).abs().max()) for m in (csi, eta, zet))
    dt = case.cfl / smax
    cp = case.params
    eps, dtau = cp.epslsm, cp.RNtimestep
    inst = [(g.ni, g.nj, g.nk, dt, dtau, eps)]

    def make_batch(**kw):
        b = LevelSetBatch(inst, RNitermax=R, btype=(1,) * 6, BigPhi=5.0, stream=stream.cuda_stream,
                          mass_correction=True, **kw)
        b.set_geometry(0, x, y, z, csi, eta, zet)
        b.set_velocity(0, q)
        b.set_phi(0, phi0)
        return b

    # ---- plain FP64 GPU path on the same grid (lsm_levelsetmethod, the
    # reference's arithmetic; no mass correction in its Sussman branch), timed
    p64 = LsmParams(epslsm=eps, delti_lsm=dt, RNitermax=R, RNtimestep=dtau, isnarrow=1, narrowcoef=4.0, BigPhi=5.0)
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    phi64, phin64 = phi0.clone(), phi0.clone()
    nc = W["compare_steps"]
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for it in range(1, nc + 1):
        if it == 2:
            e0.record()
        phin64.copy_(phi64)
        ls.levelsetmethod(g, p64, q, csi, eta, zet, aj, phi64, phin64, x, y, z, it)
    e1.record()
    torch.cuda.synchronize()
    v64 = n * (nc - 1) / (e0.elapsed_time(e1) / 1e3) / 1e9
    ls.set_stream(None)
    ls.close()
    del phi64, phin64
    torch.cuda.empty_cache()

    # ---- accuracy after the whole run: FP32 and FP64 (the same algorithm in
    # the reference's FP64 arithmetic) batches, both mass-corrected towards
    # the initial volume, NS steps each
    acc = None
    if not args.no_fp64_compare:
        b64 = make_batch(precision="fp64")
        target = float(b64.water_volume()[0, 3])
        b64.set_mass_target(0, target)
        b64.step(NS, volumes=False)
        phi64 = b64.get_phi(0, like=phi0)
        vol64 = float(b64.water_volume()[0, 3])
        b64.close()
        torch.cuda.empty_cache()
        def fp32_run():
            b32 = make_batch()
            b32.set_mass_target(0, target)
            b32.step(NS, volumes=False)
            out = b32.get_phi(0, like=phi0), float(b32.water_volume()[0, 3])
            b32.close()
            return out

        phi32, vol32 = fp32_run()
        band = phi64.abs() < 4.0 * eps
        # the same run without the FP64 stage near the interface
        os.environ["LSM_BATCH_BAND64"] = "0"
        try:
            phi32n, _ = fp32_run()
        finally:
            del os.environ["LSM_BATCH_BAND64"]
        err_no64 = float((phi32n - phi64).abs()[band].max())
        del phi32n
        acc = {"steps": NS, "band_linf_phi_err": float((phi32 - phi64).abs()[band].max()),
               "band_linf_phi_err_without_fp64_interface_terms": err_no64,
               "band": "|phi64| < 4 epslsm (6 cells)",
               "volume_rel_diff": abs(vol32 - vol64) / abs(vol64),
               "volume_drift_fp32": abs(vol32 - target) / target, "volume_drift_fp64": abs(vol64 - target) / target,
               "reference": "FP64 batch (the same algorithm in FP64, matching the FP64 oracle to 1e-12) with the same "
                            "mass correction; drift = |V(phi_T) - V(phi_0)| / V(phi_0)"}
        del phi32, phi64, band
        torch.cuda.empty_cache()

    # ---- the timed FP32 batch; the recorded segments keep the pseudo-steps'
    # adjoint coefficients when they fit in device memory (else the reverse
    # sweep recomputes them)
    need = LevelSetBatch.adjoint_bytes(n, R, NS, CK, "fp32", "store", True)
    mode = "store" if need + (8 << 30) < torch.cuda.mem_get_info()[0] else "recompute"
    b = make_batch(adjoint_mode=mode)
    target = float(b.water_volume()[0, 3])
    b.set_mass_target(0, target)
    gen = torch.Generator(device="cuda").manual_seed(0)
    wts = torch.randn(phi0.shape, generator=gen, dtype=torch.float64, device="cuda")

    def bench_step():
        # the whole run from phi0: NS steps forward with a checkpoint every CK
        # steps, then the reverse sweep (recomputing every segment but the last)
        b.set_phi(0, phi0)
        b.forward_record(NS, CK)
        b.set_grad_phi(0, wts)
        b.backward()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            bench_step()
    torch.cuda.synchronize()
    dist_barrier(world)
    lib = _lib.load()
    l0 = lib.lsm_kernel_launch_count(None)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev_index) as clocks:
        time.sleep(0.5)
        torch.cuda.synchronize()
        t_start = time.time()
        with torch.cuda.stream(stream):
            torch.cuda.nvtx.range_push("timed")   # launch-list captures filter on this range
            ev0.record(stream)
            for _ in range(args.steps):
                bench_step()
            ev1.record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        clocks.mark(t_start, time.time())
        time.sleep(0.2)
    launches = lib.lsm_kernel_launch_count(None) - l0
    dist_barrier(world)
    ms = ev0.elapsed_time(ev1)
    ms_max = dist_max(ms, world)
    value = world * n * NS * args.steps / (ms_max / 1e3) / 1e9
    shape = b.shape
    mstate = b.mass_state()[0]

    # ---- end to end through the C-ABI with host (pinned) arrays
    def pinned(a):
        a = np.asfortranarray(a)
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        return v, t

    h_phi, t1 = pinned(case.phi0)
    h_q, t2 = pinned(case.q(0.0))
    h_w, t3 = pinned(wts.cpu().numpy().T)
    h_phiT, t4 = pinned(np.zeros(g.shape))
    h_gphi, t5 = pinned(np.zeros(g.shape))
    h_gq, t6 = pinned(np.zeros((4,) + g.shape))
    keep = (t1, t2, t3, t4, t5, t6)
    e2e_steps = max(1, min(args.steps, 2))
    parts = {}

    def part(name, fn):
        t = time.perf_counter()
        fn()
        parts[name] = parts.get(name, 0.0) + (time.perf_counter() - t) * 1e3 / e2e_steps

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        part("set_phi", lambda: b.set_phi(0, h_phi))
        part("set_velocity", lambda: b.set_velocity(0, h_q))
        part("set_mass_target", lambda: b.set_mass_target(0, target))
        part("forward_record", lambda: b.forward_record(NS, CK))
        part("get_phi", lambda: b._chk(b.lib.lsm_batch_get_phi(b.h, 0, h_phiT.ctypes.data), "get_phi"))
        part("set_grad_phi", lambda: b.set_grad_phi(0, h_w))
        part("backward", lambda: b.backward())
        part("get_grad_phi0", lambda: b._chk(b.lib.lsm_batch_get_grad_phi0(b.h, 0, h_gphi.ctypes.data),
                                             "get_grad_phi0"))
        part("get_grad_velocity", lambda: b._chk(b.lib.lsm_batch_get_grad_velocity(b.h, 0, h_gq.ctypes.data),
                                                 "get_grad_velocity"))
    torch.cuda.synchronize()
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e_value = world * n * NS * e2e_steps / e2e_s / 1e9
    del keep
    b.close()
    torch.cuda.empty_cache()

    # ---- per-kernel attribution: a batch without the graph, the same schedule
    # in miniature (10 steps, a checkpoint every step: 9 plain steps, 1
    # recorded, 9 recomputed, 10 reversed -- the 0.9 : 1 : 1 proportions of
    # the full run) under the library's event timer
    b2 = make_batch(use_graph=False, autotune=False, shape=shape[0], adjoint_mode=mode)
    b2.set_mass_target(0, target)
    SA = 10
    b2.forward_record(2, 1)
    b2.set_grad_phi(0, wts)
    b2.backward()
    torch.cuda.synchronize()
    with KernelTimer() as kt:
        b2.set_phi(0, phi0)
        b2.forward_record(SA, 1)
        b2.set_grad_phi(0, wts)
        b2.backward()
        torch.cuda.synchronize()
        prof = kt.read()
    b2.close()
    peaks = load_peaks()
    roof = _roofline(prof, n, peaks, FWDADJ_BYTES, "FP32 words x 4 B per node (FP64 cell volume 8 B)")
    # whole-step roofline: algorithmic bytes of every launch of the profiled
    # schedule, per cell-step, at the measured throughput
    seg_bytes = sum(FWDADJ_BYTES[k] * n * v[0] for k, v in prof.items() if k in FWDADJ_BYTES)
    per_cell_step = seg_bytes / (float(SA) * n)
    # the same step counted by the passes of the reference's formulation
    # (each distinct array read and written once per pass): forward
    # 53 + 14R words and adjoint 131 + 32R words (which include the forward
    # recompute this schedule runs for every segment but the last), FP32
    pass_bytes = (184 + 46 * R) * 4.0
    step_roof = {"algorithmic_bytes_per_cell_step": per_cell_step,
                 "achieved_gbs": per_cell_step * value,
                 "frac": per_cell_step * value / roof["peak"],
                 "per_pass_accounting": {"bytes_per_cell_step": pass_bytes,
                                         "frac": pass_bytes * value / roof["peak"]},
                 "kernel_share_ms": {k: round(v[1], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])},
                 "note": "bytes: the launches of the profiled 10-step schedule (checkpoint every step), each "
                         "kernel's own algorithmic bytes, per cell-step"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sec, used = cpu_oracle_time(case, 1, host_threads())
        cpu = {"value": n / sec / 1e9, "unit": "Gcell-steps/s", "cores": used, "kind": "port",
               "sample": "1 physical forward step of the full %dx%dx%d grid (CPU FP64 oracle, OpenMP, %d threads; "
                         "the reference has no adjoint)" % (g.ni, g.nj, g.nk, used)}
    if rank == 0:
        line = {
            "metric": FWDADJ_METRIC % R,
            "value": value, "unit": "Gcell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (analytic 3-D free surface and solitary-wave velocity; the reference "
                                    "ships no decks)",
            "config": {"workload": FWDADJ_WORKLOAD % (g.ni, g.nj, g.nk, NS, R, CK, -(-NS // CK) - 1),
                       "nodes": n, "physical_steps_per_step": NS, "checkpoint_every": CK, "tile_shape": shape[1],
                       "adjoint_mode": mode, "adjoint_state_gb": round(need / 1e9, 1),
                       "mass_correction": {"target": target, "last_step": {"V": mstate[0], "dV_dC": mstate[1],
                                                                           "C": mstate[2]}},
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "loss": "linear, seeded N(0,1) weights on phi_T",
                       "l2": "inputs larger than L2 (phi alone %.2f GB > 129 MB)" % (n * 4 / 1e9)},
            "roofline": roof,
            "step_roofline": step_roof,
            "cpu_baseline": cpu,
            "fp64_gpu_path": {"value": v64, "unit": "Gcell-steps/s", "sample": "%d forward steps of the same grid, "
                              "lsm_levelsetmethod (reference FP64 arithmetic)" % (nc - 1),
                              "speedup_fp32_fwd_adj": value / v64},
            "accuracy_vs_fp64": acc,
            "e2e": {"value": e2e_value, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 8 * n * (1 + 4 + 1) + 8,
                    "d2h_bytes_per_step": 8 * n * (1 + 1 + 4), "steps": e2e_steps,
                    "ms_per_call": {k: round(v, 1) for k, v in parts.items()}},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
            "kernel_times_ms": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in prof.items()},
        }
        print(json.dumps(line))


def run_fp64(args):
    import torch
    from nslsm import LevelSet
    from nslsm._lib import KernelTimer

    rank, world = dist_setup(args.gpus)
    dev_index = torch.cuda.current_device()
    W = workload(args)
    scheme = FP64_SCHEME[args.workload]
    case = make_case(W["ni"], W["nj"], W["nk"], W["reinit_iters"], scheme)
    case.redistance_iters = W["redistance"]
    n = case.grid.n
    ls = LevelSet(device=dev_index)
    ls.set_stream(torch.cuda.current_stream().cuda_stream)
    d = prepare_device(case, ls, torch)
    phi = d["phi"]
    phin = phi.clone()

    def step(it):
        phin.copy_(phi)
        ls.levelsetmethod(d["g"], d["p"], d["q"], d["csi"], d["eta"], d["zet"], d["aj"], phi, phin, d["x"],
                          d["y"], d["z"], it)

    for it in range(1, args.warmup + 1):
        step(it)
    torch.cuda.synchronize()
    dist_barrier(world)
    l0 = ls.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev_index) as clocks:
        time.sleep(0.5)          # let the sampler start before the timed region
        torch.cuda.synchronize()
        t_start = time.time()
        ev0.record()
        for it in range(args.warmup + 1, args.warmup + args.steps + 1):
            step(it)
        ev1.record()
        torch.cuda.synchronize()
        clocks.mark(t_start, time.time())
        time.sleep(0.2)
    launches = ls.launches - l0
    dist_barrier(world)
    ms = ev0.elapsed_time(ev1)
    ms_max = dist_max(ms, world)
    value = world * n * args.steps / (ms_max / 1e3) / 1e9

    # per-kernel attribution (a separate pass with the event timer on)
    with KernelTimer() as kt:
        for it in range(1, min(args.steps, 5) + 1):
            step(it)
        torch.cuda.synchronize()
        prof = kt.read()
    roof = roofline_from_profile(prof, n, load_peaks())

    # end-to-end through the C-ABI with pinned host arrays
    def pinned(a):
        a = np.asfortranarray(a)
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        v = t.numpy().reshape(a.shape, order="F")
        v[...] = a
        return v, t

    keep = []
    host = {}
    for k in ("q", "csi", "eta", "zet", "aj", "x", "y", "z"):
        arr = d[k].cpu().numpy().T
        host[k], t = pinned(arr)
        keep.append(t)
    hphi, t1 = pinned(phi.cpu().numpy().T)
    hphin, t2 = pinned(phi.cpu().numpy().T)
    keep += [t1, t2]
    e2e_steps = max(2, min(args.steps, 10))
    ls.set_stream(None)
    for it in range(1, 2):
        ls.levelsetmethod(d["g"], d["p"], host["q"], host["csi"], host["eta"], host["zet"], host["aj"], hphi, hphin,
                          host["x"], host["y"], host["z"], it)
    torch.cuda.synchronize()
    dist_barrier(world)
    t0 = time.perf_counter()
    for it in range(1, e2e_steps + 1):
        hphin[...] = hphi
        ls.levelsetmethod(d["g"], d["p"], host["q"], host["csi"], host["eta"], host["zet"], host["aj"], hphi, hphin,
                          host["x"], host["y"], host["z"], it)
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e_value = world * n * e2e_steps / e2e_s / 1e9
    h2d = 8 * n * (4 + 9 + 1 + 1 + 1 + 3)
    d2h = 8 * n + 32

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = host_threads()
        if scheme == 2:
            # an eighth of the grid keeps the oracle's step within the bench's minutes
            sg = (W["ni"] // 2, W["nj"] // 2, W["nk"] // 2)
            sample = make_case(sg[0], sg[1], sg[2], W["reinit_iters"], scheme)
            sec, used = cpu_oracle_time(sample, 1, threads)
            cpu = {"value": sample.grid.n / sec / 1e9, "unit": "Gcell-steps/s", "cores": used, "kind": "port",
                   "sample": "1 physical step of the same case on %dx%dx%d nodes (FP64 oracle, OpenMP, %d "
                             "threads; the Newton solve serial)" % (sg + (used,))}
        else:
            sample = make_case(W["ni"], W["nj"], W["nk"], W["reinit_iters"], scheme)
            sec, used = cpu_oracle_time(sample, 1, threads)
            cpu = {"value": n / sec / 1e9, "unit": "Gcell-steps/s", "cores": used, "kind": "port",
                   "sample": "1 physical step of the full 256x128x96 workload (FP64 oracle, OpenMP, %d threads, "
                             "phi0 not redistanced)" % used}
    if rank == 0:
        line = {
            "metric": FP64_METRIC[scheme],
            "value": value, "unit": "Gcell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (analytic solitary-wave workload; the reference ships no decks)",
            "config": {"workload": "solitary_wave curvilinear %dx%dx%d, CFL 0.4, WENO3+TVD-RK3, %d reinit "
                                   "pseudo-steps/step (%s), volume each step"
                                   % (W["ni"], W["nj"], W["nk"], W["reinit_iters"], FP64_REINIT[scheme]),
                       "nodes": n, "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (working set %.2f GB > 129 MB)" % (n * 8 * 30 / 1e9)},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "Gcell-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
            "kernel_times_ms": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in prof.items()},
        }
        print(json.dumps(line))
    ls.close()


# ---------------------------------------------------------- reference arm
def run_reference(args):
    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    if rank != 0:
        return
    if args.workload == "batched":
        return run_reference_batched(args, world)
    if args.workload == "fwdadj":
        return run_reference_fwdadj(args, world)
    if args.workload == "adjcheck":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint"}))
        return
    W = workload(args)
    scheme = FP64_SCHEME[args.workload]
    if scheme == 2 and not args.grid:
        # an eighth of the grid keeps the oracle's steps within the bench's minutes
        W["ni"], W["nj"], W["nk"] = W["ni"] // 2, W["nj"] // 2, W["nk"] // 2
    case = make_case(W["ni"], W["nj"], W["nk"], W["reinit_iters"], scheme)
    threads = host_threads()
    # warm-up (page-in, thread pool) then timed steps, each a full physical step
    cpu_oracle_time(case, max(1, min(args.warmup, 1)), threads)
    steps = max(1, min(args.steps, 3))
    sec, used = cpu_oracle_time(case, steps, threads)
    v = case.grid.n / sec / 1e9
    line = {
        "impl": "reference",
        "metric": FP64_METRIC[scheme],
        "value": v, "unit": "Gcell-steps/s", "n_gpus": world, "steps": steps, "warmup": 1,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": "solitary_wave curvilinear %dx%dx%d, %d reinit pseudo-steps/step"
                                        " (%s)" % (W["ni"], W["nj"], W["nk"], W["reinit_iters"],
                                                   FP64_REINIT[scheme])},
        "cpu_baseline": {"value": v, "unit": "Gcell-steps/s", "cores": used, "kind": "port",
                         "sample": "%d full physical steps; CPU FP64 restatement of the reference (the Fortran/MPI "
                                   "original cannot be built here: no Fortran compiler)" % steps},
        "e2e": {"value": v, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_reference_batched(args, world):
    """The CPU FP64 restatement of the reference (all host threads) on the
    batched workload: each timed step advances a rotating group of 8 of the
    64 instances by one physical step (bounded sample)."""
    from nslsm import configs
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    threads = host_threads()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle as O
    O.build()
    orc = O.Oracle(omp=True)
    R = BATCH["reinit_iters"]
    insts = configs.batched_instances(BATCH["n_inst"], BATCH["lo"], BATCH["hi"], BATCH["seed"], BATCH["cfl"])
    prepared = []
    for it in insts:
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = orc.mg_metrics(g, it.x, it.y, it.z)
        p = O.make_params(epslsm=it.eps, delti_lsm=it.time_step(csi, eta, zet), RNitermax=R, RNtimestep=it.dtau,
                          BigPhi=5.0)
        prepared.append((it, g, p, csi, eta, zet, aj))

    def one(group, s):
        nodes = 0
        for it, g, p, csi, eta, zet, aj in group:
            orc.levelsetmethod(g, p, it.q, csi, eta, zet, aj, it.phi0, it.phi0, it.x, it.y, it.z, s)
            nodes += it.grid.n
        return nodes

    one(prepared[:2], 1)
    steps = max(1, min(args.steps, 3))
    nodes, t0 = 0, time.perf_counter()
    for s in range(steps):
        grp = [prepared[(8 * s + q) % len(prepared)] for q in range(8)]
        nodes += one(grp, s + 1)
    sec = time.perf_counter() - t0
    v = nodes / sec / 1e9
    line = {
        "impl": "reference",
        "metric": "Gcell-steps/s (batched FP32 level-set step, forward: WENO3-RK3 + %d reinit pseudo-steps + "
                  "FP64 volume, 64 uneven instances)" % R,
        "value": v, "unit": "Gcell-steps/s", "n_gpus": world, "steps": steps, "warmup": 1,
        "ms_per_step": sec / steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "batched_instances 64 x U{32..96}^3, %d reinit pseudo-steps/step" % R},
        "cpu_baseline": {"value": v, "unit": "Gcell-steps/s", "cores": orc.threads, "kind": "port",
                         "sample": "%d steps, each one physical step of 8 of the 64 instances (%d nodes in total); "
                                   "CPU FP64 restatement of the reference (the Fortran/MPI original cannot be built "
                                   "here: no Fortran compiler)" % (steps, nodes)},
        "e2e": {"value": v, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_adjcheck(args):
    """The adjoint configuration: 128^3 unit box, sphere r = 0.15 at (0.35,
    0.35, 0.35), LeVeque deformation field (frozen at t = 0 over the run),
    50 steps of WENO3-RK3 + 5 reinitialisation pseudo-steps, eps = 1.5 h;
    loss = sum (H_eps(phi_T) - H_eps(phi_target))^2 with phi_target from a
    run with the velocity scaled by 1.05; gradients with respect to phi0
    and the velocity by the hand-written adjoint with a checkpoint every 10
    steps, FP64 then FP32.  Checks: central differences of the FP64 forward
    along 16 seeded directions (step 1e-6; a direction whose difference
    quotient changes between steps h and h/2 crossed a branch point and is
    not scored), the FP32 gradient against the FP64 one, and the FP64 batch
    gradient against the FP64 torch tape on a 32^3 copy (tests/lsm_tape.py).
    value = the largest relative error against central differences."""
    import torch
    from nslsm import LevelSet, configs
    from nslsm.batch import LevelSetBatch
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import lsm_tape as TAPE

    NSTEPS, CKPT, R = 50, 10, 5

    def H(p, e):
        return torch.where(p < -e, torch.zeros_like(p), torch.where(p > e, torch.ones_like(p),
                           0.5 * (1.0 + p / e + torch.sin(np.pi * p / e) / np.pi)))

    def dH(p, e):
        return torch.where(p.abs() > e, torch.zeros_like(p), (1.0 + torch.cos(np.pi * p / e)) / (2.0 * e))

    def setup(n):
        case = configs.sphere_deformation(n, reinit_iters=R)
        g = case.grid
        ls = LevelSet(device=0)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()  # noqa: E731
        x, y, z = dev(case.x), dev(case.y), dev(case.z)
        csi, eta, zet, aj = ls.mg_metrics(g, x, y, z)
        q = dev(case.q(0.0))
        smax = max(float((m * q[..., 1:4]).sum(-1).abs().max()) for m in (csi, eta, zet))
        dt = case.cfl / smax
        ls.close()
        return dict(case=case, g=g, x=x, y=y, z=z, csi=csi, eta=eta, zet=zet, q=q, phi0=dev(case.phi0), dt=dt)

    def batch(S, prec):
        c = S["case"]
        b = LevelSetBatch([(S["g"].ni, S["g"].nj, S["g"].nk, S["dt"], c.params.RNtimestep, c.params.epslsm)],
                          RNitermax=R, btype=(1,) * 6, BigPhi=5.0, precision=prec, autotune=False)
        b.set_geometry(0, S["x"], S["y"], S["z"], S["csi"], S["eta"], S["zet"])
        return b

    def forward(b, phi0, q):
        b.set_velocity(0, q)
        b.set_phi(0, phi0)
        b.step(NSTEPS, volumes=False)
        return b.get_phi(0, like=phi0)

    def adjoint(b, S, phi0, q, target):
        eps = S["case"].params.epslsm
        b.set_velocity(0, q)
        b.set_phi(0, phi0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.forward_record(NSTEPS, CKPT)
        phiT = b.get_phi(0, like=phi0)
        seed = 2.0 * (H(phiT, eps) - H(target, eps)) * dH(phiT, eps)
        b.set_grad_phi(0, seed)
        b.backward()
        gphi, gq = b.get_grad_phi0(0, like=phi0), b.get_grad_velocity(0, like=phi0)
        torch.cuda.synchronize()
        return gphi, gq, time.perf_counter() - t0

    S = setup(128)
    eps = S["case"].params.epslsm
    b64 = batch(S, "fp64")
    target = forward(b64, S["phi0"], 1.05 * S["q"])
    loss = lambda phi0, q: float(((H(forward(b64, phi0, q), eps) - H(target, eps)) ** 2).sum())  # noqa: E731
    gphi, gq, t64 = adjoint(b64, S, S["phi0"], S["q"], target)
    # the forward map is piecewise smooth: the band test |phi| < eps of the
    # sign field and the upwind / Godunov selections switch along the way, so
    # a perturbation crosses some switches with a probability that grows with
    # the step; both the config's step and a smaller one are reported
    fd = {}
    for h in (1e-6, 1e-8):
        gen = torch.Generator(device="cuda").manual_seed(7)
        worst, scored, skipped, rows = 0.0, 0, 0, []
        for d in range(16):
            v = torch.randn(S["phi0"].shape if d % 2 == 0 else S["q"].shape, generator=gen, dtype=torch.float64,
                            device="cuda")
            if d % 2 == 0:
                f = lambda t: loss(S["phi0"] + t * v, S["q"])  # noqa: E731
                an = float((gphi * v).sum())
            else:
                v[..., 0] = 0.0
                f = lambda t: loss(S["phi0"], S["q"] + t * v)  # noqa: E731
                an = float((gq * v).sum())
            fd1 = (f(h) - f(-h)) / (2 * h)
            fd2 = (f(0.5 * h) - f(-0.5 * h)) / h
            rows.append([d, an, fd1, fd2])
            if abs(fd1 - fd2) > 1e-3 * max(abs(fd1), abs(fd2), 1e-300):
                skipped += 1
                continue
            scored += 1
            worst = max(worst, abs(an - fd1) / max(abs(fd1), abs(an), 1e-300))
        fd["%g" % h] = {"directions_scored": scored, "directions_skipped": skipped,
                        "max_rel_err": worst if scored else None, "directions": rows}
    b64.close()
    b32 = batch(S, "fp32")
    g32phi, g32q, t32 = adjoint(b32, S, S["phi0"], S["q"], target)
    b32.close()
    rel = lambda a, r: float((a - r).norm() / r.norm())  # noqa: E731
    fp32_vs_fp64 = {"grad_phi0": rel(g32phi, gphi), "grad_q": rel(g32q, gq)}

    # FP64 torch tape on a 32^3 copy
    T = setup(32)
    bt = batch(T, "fp64")
    tgt = forward(bt, T["phi0"], 1.05 * T["q"])
    gp, gqq, _ = adjoint(bt, T, T["phi0"], T["q"], tgt)
    bt.close()
    M = [m[..., c].contiguous() for m in (T["csi"], T["eta"], T["zet"]) for c in range(3)]
    p0 = T["phi0"].clone().requires_grad_(True)
    qq = T["q"].clone().requires_grad_(True)
    cp = T["case"].params
    out = TAPE.run(p0, qq, M, T["dt"], cp.RNtimestep, cp.epslsm, R, NSTEPS)
    ((H(out, cp.epslsm) - H(tgt, cp.epslsm)) ** 2).sum().backward()
    tape = {"grad_phi0": rel(gp, p0.grad), "grad_q": rel(gqq, qq.grad)}
    n = S["g"].n
    line = {
        "metric": "adjoint check: largest relative error of the FP64 adjoint against central differences "
                  "(16 seeded directions, step 1e-6)",
        "value": fd["1e-06"]["max_rel_err"], "unit": "relative error", "n_gpus": 1, "steps": NSTEPS, "warmup": 0, "ms_per_step": None,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic sphere and deformation field)",
        "config": {"workload": "sphere in the deformation field, 128^3, %d steps, %d reinit pseudo-steps/step, "
                               "Heaviside loss against a 1.05x-velocity target, checkpoint every %d steps"
                               % (NSTEPS, R, CKPT), "nodes": n},
        "fd": dict(fd, bar=1e-4, skip_rule="difference quotients at h and h/2 differ by more than 1e-3"),
        "fp32_vs_fp64": fp32_vs_fp64,
        "tape_32cubed": tape,
        "adjoint_seconds": {"fp64": t64, "fp32": t32},
        "fwdadj_gcell_steps_per_s": {"fp64": n * NSTEPS / t64 / 1e9, "fp32": n * NSTEPS / t32 / 1e9},
    }
    print(json.dumps(line))


def run_reference_fwdadj(args, world):
    """The CPU FP64 restatement of the reference (all host threads) on the
    large free-surface grid: each timed step is one physical forward step of
    the whole grid (the reference has no adjoint)."""
    from nslsm import configs
    W = dict(FWDADJ)
    if args.grid:
        W["ni"], W["nj"], W["nk"] = (int(v) for v in args.grid.lower().split("x"))
    R = W["reinit_iters"]
    case = configs.large_free_surface(W["ni"], W["nj"], W["nk"], reinit_iters=R)
    threads = host_threads()
    # a physical step of the whole grid takes a few seconds on the box's 16
    # cores: the requested counts, capped so the run stays within minutes
    steps = max(1, min(args.steps if args.steps else 10, 10))
    warm = max(0, min(args.warmup, 3))
    sec, used = cpu_oracle_time(case, steps, threads, warm)
    v = case.grid.n / sec / 1e9
    NS, CK = W["nsteps"], min(W["ckpt"], W["nsteps"])
    line = {
        "impl": "reference",
        "metric": FWDADJ_METRIC % R,
        "value": v, "unit": "Gcell-steps/s", "n_gpus": world, "steps": steps, "warmup": warm,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": FWDADJ_WORKLOAD % (W["ni"], W["nj"], W["nk"], NS, R, CK, -(-NS // CK) - 1),
                   "nodes": case.grid.n,
                   "timed": "one physical forward step of the whole grid per step (the reference has no adjoint "
                            "and no mass correction in its Sussman branch)"},
        "cpu_baseline": {"value": v, "unit": "Gcell-steps/s", "cores": used, "kind": "port",
                         "sample": "%d physical forward steps of the whole grid; CPU FP64 restatement of the "
                                   "reference (the Fortran/MPI original cannot be built here: no Fortran compiler); "
                                   "the reference has no adjoint, so forward only" % steps},
        "e2e": {"value": v, "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def workload(args):
    W = dict(WORKLOAD)
    if args.grid:
        W["ni"], W["nj"], W["nk"] = (int(v) for v in args.grid.lower().split("x"))
    return W


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 3 for fwdadj, else 30)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", default=None, help="NIxNJxNK instead of the workload's grid (profiling runs)")
    ap.add_argument("--workload", choices=["fwdadj", "batched", "fp64", "sussman", "hybrid", "adjcheck"],
                    default="fwdadj")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--n-inst", type=int, default=None, help="instances of the batched workload (profiling runs)")
    ap.add_argument("--segment", type=int, default=None,
                    help="checkpoint interval of the fwdadj workload (profiling runs)")
    ap.add_argument("--nsteps", type=int, default=None,
                    help="physical steps of the fwdadj workload's run (profiling runs)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 3 if args.workload == "fwdadj" else 30
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
