"""Throughput of the RK3 substep on one GB300 (or N replicas, one per GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload C1] [--form both|fp64|mixed] [--nonlin products|triads]

Metric: Mpts*substeps/s = N1*N2*ny mode-points per RK3 substep, 3 substeps per step.
`value` is the headline form (mixed when its velocity error against the FP64 form
stays within 1e-5, else FP64) with the state resident in HBM; `e2e` is the same
metric through the C ABI with the state copied from pinned host memory and back
every step. The path does not shard (replicas only): with N > 1 every rank runs its
own channel and `value` sums the replicas. `--nonlin triads` runs the as-run
triad-list nonlinear term (complete lists, threshold 0) instead of the products.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpts·RK3-substeps/s on 1 GB300, mixed vs FP64 at ≤1e-5 rel err; CPU ref beside"
UNIT = "Mpts*substeps/s"


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return ws, rank, local, pg


def reduce_max(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() and pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled during the timed region: through
    NVML (libnvidia-ml, read-only queries) every 10 ms from a thread when the library loads,
    else nvidia-smi every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # clock-event reason bits of NVML
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
            "hw_power_brake_slowdown": 0x80}

    def __init__(self, gpu_index: int):
        self.p = self.thread = None
        self.samples, self.reason_bits, self.max_mhz = [], 0, None
        if self._nvml_start(gpu_index):
            return
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def _nvml_start(self, gpu_index: int) -> bool:
        import ctypes
        import threading
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return False
            h = ctypes.c_void_p()
            ok = False
            try:  # the device this process uses, by PCI bus id (CUDA and NVML numbering may differ)
                import torch
                pr = torch.cuda.get_device_properties(gpu_index)
                bus = b"%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
                ok = nv.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(h)) == 0
            except Exception:
                ok = False
            if not ok and nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu_index), ctypes.byref(h)) != 0:
                return False
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
        except (OSError, AttributeError):
            return False
        self.stop_flag = threading.Event()

        def run():
            clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
            while not self.stop_flag.is_set():
                if nv.nvmlDeviceGetClockInfo(h, ctypes.c_int(1), ctypes.byref(clk)) == 0:
                    self.samples.append(float(clk.value))
                if reasons_fn(h, ctypes.byref(rs)) == 0:
                    self.reason_bits |= rs.value
                self.stop_flag.wait(0.01)

        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        return True

    def stop(self) -> dict:
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join(timeout=5)
            sm = sorted(self.samples)
            reasons = sorted(n for n, b in self.BITS.items() if self.reason_bits & b)
            return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": self.max_mhz, "reasons": reasons,
                    "samples": len(sm), "source": "nvml"}
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [l.strip().split(",") for l in self.f.read().splitlines() if l.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi"}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    """Per-launch DRAM bytes of a kernel on a workload from the committed ncu summary
    (profiles/ncu_traffic_C1.txt: `workload kernel form bytes_per_launch` lines)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic_C1.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            f = line.split()
            if len(f) >= 4 and not line.startswith("#"):
                try:
                    out[(f[0], f[1], f[2])] = float(f[3])
                except ValueError:
                    pass
    return out


def plane_views(s):
    """(u planes, v planes, N1h, G2, modes per plane) of each plane class: wall-band
    planes, then core planes (multiblock only)."""
    nuI, nvI = s.nyu - 2, s.nyv - 2
    if not s.multiblock:
        return [(nuI, nvI, s.N1 // 2 + 1, s.G2, s.ncols)]
    d = s.dny
    ju = np.arange(1, s.nyu - 1) - d
    jv = np.arange(1, s.nyv - 1) - d
    fu = int(((ju <= s.N[3, 1]) | (ju > s.N[3, 2])).sum())
    fv = int(((jv <= s.N[2, 1]) | (jv > s.N[2, 2])).sum())
    return [(fu, fv, s.N1 // 2 + 1, s.G2, s.ncols),
            (nuI - fu, nvI - fv, s.N1c // 2 + 1, s.G2c, (s.N1c // 2 + 1) * s.N2c)]


def column_levels(s, grid: int) -> int:
    """Sum over the solve segments of (levels of `grid`): long columns span the channel,
    short columns their two wall bands."""
    tot = 0
    for b in (1, 2, 3):
        lo, hi = s.band_levels(b, grid)
        tot += len(s.band_cols(b)) * (hi - lo + 1)
    return tot


def algorithmic_bytes(s, kernel: str, form: str, nterms: int = 0, ib: bool = True) -> float:
    """Compulsory HBM bytes of one substep's launches of a kernel: every input and
    output element once. Spectral fields are complex128; the transform intermediates
    and the forward z pass's outputs are complex128 in the FP64 form and complex64 in
    the mixed form. The inverse z pass reads each field on its own planes (u and w on
    the u planes, v on the v planes); the staggered interpolation's neighbour planes are
    the same elements again (a plane at each band edge aside) and count once. The triad kernel
    reads one 4-byte term per complex multiply-add (`nterms` per substep), the three
    velocities of every interior plane and writes five (u planes) / three (v planes)
    products in the transform precision."""
    vs = 16 if form == "fp64" else 8
    z = 16
    tot = 0.0
    for nuI, nvI, N1h, G2, ncv in plane_views(s):
        A = (nuI + nvI) * 3 * G2 * N1h * vs
        B = (4 * nuI + 2 * nvI) * N1h * G2 * vs
        if kernel == "k_zinv_nl":
            tot += (2 * nuI + nvI) * ncv * z + A
        elif kernel == "k_xpass_nl":
            tot += A + B
        elif kernel == "k_zfwd_nl":
            tot += B + (nuI + nvI) * 3 * ncv * vs
    if kernel == "k_xpass_nl" and ib and s.dny > 0 and s.p.ib_enable and s.p.geometry_type == 2:
        # physical planes of the immersed-boundary levels (and the two tip levels) captured
        # for the forcing: 3 fields, in the transform precision
        tot += (4 * s.dny + 2) * 3 * s.G1 * s.G2 * (8 if form == "fp64" else 4)
    if kernel in ("k_zinv_nl", "k_xpass_nl", "k_zfwd_nl"):
        return tot
    # the solves: the FP64 state read and written (u and w / v) and p read, the nonlinear
    # term N read and written, the z pass's output and the y-flux read, in the transform
    # precision (FP64 form: 13 / 7 complex128 per column level)
    if kernel == "k_helm_uw":
        return column_levels(s, 2) * (4 * z + z + 2 * 4 * vs)
    if kernel == "k_helm_v":
        return column_levels(s, 1) * (2 * z + z + 4 * vs)
    if kernel == "k_press":
        return column_levels(s, 2) * z * 8
    if kernel == "k_triad":
        ncol = (s.N1 // 2 + 1) * s.N2
        nu, nv = s.nyu - 2, s.nyv - 2
        return nterms * 4 + (nu + nv) * 3 * ncol * z + (5 * nu + 3 * nv) * ncol * vs
    return float("nan")


def triad_lists(args, s):
    if args.nonlin != "triads":
        return None
    from rnl_multiblock_nofft_gb300.triads import TriadLists
    return TriadLists.complete(s)


def triad_terms(s, tl) -> int:
    """Multiply-adds of complex values per substep in the triad sums: every list
    triad counts twice (both z-signs) except those with ka + kp = 0."""
    from rnl_multiblock_nofft_gb300.triads import U_TYPES, V_TYPES, plane_files
    fu, fv = plane_files(s)
    cache = {}
    n = 0
    for files, types in ((fu[1:-1], U_TYPES), (fv[1:-1], V_TYPES)):
        for j in files:
            for t in types:
                a = tl.files[int(j)][t - 1]
                k = id(a)
                if k not in cache:
                    cache[k] = 2 * len(a) - int(((a[:, 1].astype(int) + a[:, 3]) == 0).sum())
                n += cache[k]
    return n


def error_by_steps(s, tl, ic, sc0, mb, counts):
    """Relative L2 error of the mixed form against the FP64 form, per field, after each of
    `counts` steps from the same initial state (untimed)."""
    import numpy as np
    from rnl_multiblock_nofft_gb300.native import GpuChannel
    ref, out = {}, {}
    for form in ("fp64", "mixed"):
        g = GpuChannel(s, form, triads=tl)
        if mb:
            g.upload_bands(ic)
        else:
            g.upload_state(*ic)
        g.set_scalars(**sc0)
        done = 0
        for n in sorted(counts):
            g.step(n - done)
            done = n
            g.synchronize()
            st = [a for b in (1, 2, 3) for a in g.download_bands()[b]] if mb else g.download_state()
            if form == "fp64":
                ref[n] = st
                continue
            e = {}
            for i, f in enumerate(("u1", "u2", "u3", "p")):
                a = np.concatenate([x.ravel() for x in ref[n][i::4]])
                b = np.concatenate([x.ravel() for x in st[i::4]])
                e[f] = float(np.linalg.norm(b - a) / np.linalg.norm(a))
            del ref[n]
            out[str(n)] = e
        g.close()
    return out


def oracle_initial_state(o, s):
    from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_field_bands
    if s.multiblock:
        o.set_bands(initial_field_bands(s, 1000))
    else:
        o.set_state(*initial_field(s, 1000))


def run_reference(args, ws, rank):
    """The reference's CPU path on the host cores: the Fortran/MPI reference cannot
    be built here (no Fortran compiler), so its restatement (the oracle) runs on
    every host thread; each timed step is one RK3 substep of the workload."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup
    s = workload_setup(args.workload)
    cores = os.cpu_count() or 1
    o = Oracle(s, threads=cores, triads=triad_lists(args, s))
    oracle_initial_state(o, s)
    o.set_scalars(**initial_scalars(s))
    k = 0
    for _ in range(args.warmup):
        o.substep(k % 3 + 1)
        k += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.substep(k % 3 + 1)
        k += 1
    dt = time.perf_counter() - t0
    pts = s.mode_points()
    val = pts * args.steps / dt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded perturbed laminar channel)",
            "config": {"workload": f"{args.workload}: {workload_desc(args.workload)}", "form": "fp64",
                       "step": "one RK3 substep"},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} RK3 substeps of {args.workload} on the CPU oracle "
                                       f"(the Fortran reference cannot be compiled on this image)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_desc(name):
    from rnl_multiblock_nofft_gb300.workloads import WORKLOADS
    return WORKLOADS[name]["desc"]


def cpu_baseline(s, budget_s: float = 20.0, triads=None):
    """Oracle on the host cores, bounded: RK3 substeps of the same workload until
    ~budget_s of CPU work (at least one)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars
    cores = os.cpu_count() or 1
    o = Oracle(s, threads=cores, triads=triads)
    oracle_initial_state(o, s)
    o.set_scalars(**initial_scalars(s))
    n, t0 = 0, time.perf_counter()
    while True:
        o.substep(n % 3 + 1)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 6 or (n >= 1 and el * (n + 1) / n > 2 * budget_s):
            break
    return {"value": s.mode_points() * n / el / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} RK3 substeps of the same workload on the CPU oracle, {cores} OpenMP threads, {el:.1f} s"}


def time_steps(g, steps, torch):
    stream = torch.cuda.ExternalStream(g.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = g.kernel_launches()
    e0.record(stream)
    g.step(steps)
    e1.record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), g.kernel_launches() - l0


def run_ensemble(args, ws, rank, pg, torch, np):
    """Config 3: 64 independent channels of uneven sizes, one graph launch per RK3
    step of all of them (lh_batch_*). Points = the sum over channels."""
    from rnl_multiblock_nofft_gb300.native import GpuBatch, GpuChannel
    from rnl_multiblock_nofft_gb300.workloads import ensemble_setups, initial_field, initial_scalars
    setups = ensemble_setups(64, seed=2000 + 1000 * rank)
    pts = sum(s.mode_points() for s in setups)
    forms = ["fp64", "mixed"] if args.form == "both" else [args.form]
    res = {}
    for form in forms:
        chans = []
        for c, s in enumerate(setups):
            g = GpuChannel(s, form)
            g.upload_state(*initial_field(s, 2000 + c))
            g.set_scalars(**initial_scalars(s))
            chans.append(g)
        b = GpuBatch(chans)
        b.step(args.warmup)
        b.synchronize()
        barrier(pg)
        stream = torch.cuda.ExternalStream(b.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = sum(g.kernel_launches() for g in chans)
        e0.record(stream)
        b.step(args.steps)
        e1.record(stream)
        b.synchronize()
        torch.cuda.synchronize()
        ms = reduce_max(pg, e0.elapsed_time(e1))
        res[form] = {"value": ws * pts * 3 * args.steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / args.steps,
                     "launches": sum(g.kernel_launches() for g in chans) - l0}
        b.close()
        for g in chans:
            g.close()
    head = "mixed" if "mixed" in res else forms[0]
    line = {"metric": METRIC, "value": res[head]["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res[head]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "fp64" else "f32 transforms/products and Helmholtz solves; f64 state, (0,0) mode, pressure and flux correction",
            "data": "synthetic ensemble (seeded grids, Re_tau, textures and fields)",
            "config": {"workload": "C3: 64 channels, N in {32,48,64,96}, ny in {97,129,153}, Re_tau 120-300, posts",
                       "form": head, "mode_points_per_substep": pts, "launch": "one CUDA graph per step"},
            "gpu_launches": res[head]["launches"], "forms": res}
    if rank == 0:
        print(json.dumps(line), flush=True)


def e2e_run(s, form, tl, ic, icb, sc0, steps, ws, pg, torch, np):
    """The metric through the C ABI: every step's state copied in from pinned host memory and
    the result copied back (queued lh_upload_state_async / lh_download_state_async, per band
    for multiblock channels), timed on the host clock around the whole chain."""
    from rnl_multiblock_nofft_gb300.native import GpuChannel
    mb = icb is not None
    g = GpuChannel(s, form, triads=tl)
    shapes = [sh for b in (1, 2, 3) for sh in s.band_shapes(b)] if mb else list(g.shapes)
    pin = lambda sh: torch.empty(tuple(sh) + (2,), dtype=torch.float64, pin_memory=True).numpy().view(np.complex128)[..., 0]
    pinned = [pin(sh) for sh in shapes]
    for dst, src in zip(pinned, ic):
        dst[...] = src
    pinned_out = [pin(sh) for sh in shapes]
    if mb:
        g.upload_bands({b: pinned[4 * (b - 1):4 * b] for b in (1, 2, 3)})
    else:
        g.upload_state(*pinned)
    g.set_scalars(**sc0)
    bin_ = {b: pinned[4 * (b - 1):4 * b] for b in (1, 2, 3)} if mb else None
    bout = {b: pinned_out[4 * (b - 1):4 * b] for b in (1, 2, 3)} if mb else None

    def io_step():
        if mb:
            g.upload_bands_async(bin_)
            g.step(1)
            g.download_bands_async(bout)
        else:
            g.upload_state_async(*pinned)
            g.step(1)
            g.download_state_async(pinned_out)

    # warm-up: the first queued copy creates the staging buffers, streams and events
    for _ in range(2):
        io_step()
    g.synchronize()
    barrier(pg)
    nb = sum(a.nbytes for a in pinned)
    t0 = time.perf_counter()
    for _ in range(steps):
        io_step()
    g.synchronize()
    e2e_s = reduce_max(pg, time.perf_counter() - t0)
    g.close()
    return {"value": ws * s.mode_points() * 3 * steps / e2e_s / 1e6, "unit": UNIT,
            "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb}


def kernel_roofline(s, kern, form, tl, peak, peak_kind, workload):
    """Roofline of the kernel with the largest share of the step (live per-kernel CUDA-event
    times of one eager step): algorithmic bytes per launch / average launch time."""
    dom = max(kern.items(), key=lambda kv: kv[1][1])
    dname, (dlaunch, dms) = dom
    alg_step = 3 * algorithmic_bytes(s, dname, form, triad_terms(s, tl) if tl is not None else 0)
    achieved = alg_step / (dms * 1e-3) / 1e9
    alg = alg_step / dlaunch
    if not math.isfinite(achieved):  # a kernel without an algorithmic byte count
        achieved = alg = None
    step_total = sum(v[1] for v in kern.values())
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak if achieved is not None else None,
           "traffic": traffic_table().get((workload, dname, form)), "kernel": dname,
           "kernel_share": dms / step_total, "avg_launch_ms": dms / dlaunch,
           "algorithmic_bytes_per_launch": alg, "peak_source": peak_kind}
    if dname == "k_xpass_nl":  # the same without the captured physical planes of the immersed levels
        ab = 3 * algorithmic_bytes(s, dname, form, ib=False) / (dms * 1e-3) / 1e9
        out["frac_A_B_only"] = ab / peak
    if dname == "k_press":
        out["limiter"] = "FP64 pipe: the FP64 state updates and sweeps (ncu: FP64 pipe ~83 % busy, DRAM ~46 %)"
    # the other large kernels against the same HBM roofline (live CUDA-event times)
    others = {}
    for name, (nl, ms) in sorted(kern.items(), key=lambda kv: -kv[1][1])[:6]:
        ab = 3 * algorithmic_bytes(s, name, form, triad_terms(s, tl) if tl is not None else 0)
        if name != dname and math.isfinite(ab) and ms > 0:
            others[name] = {"frac": ab / (ms * 1e-3) / 1e9 / peak, "share": ms / step_total}
    out["others"] = others
    return out


def step_roofline(s, form, ms_per_step, peak, peak_kind):
    """The whole step against the HBM roofline with fixed algorithmic bytes per mode-point and
    substep: 960 B (FP64 form) / 736 B (mixed form), plus 210 B x (immersed levels / ny) with
    posts."""
    b = 960.0 if form == "fp64" else 736.0
    ib = 210.0 * (2 * s.dny) / s.p.ny if (s.dny > 0 and s.p.geometry_type == 2) else 0.0
    per_s = s.mode_points() * 3 / (ms_per_step * 1e-3)
    ach = (b + ib) * per_s / 1e9
    return {"bytes_per_mode_point": b, "ib_bytes_per_mode_point": ib, "achieved": ach, "peak": peak,
            "unit": "GB/s", "frac": ach / peak, "frac_without_ib": b * per_s / 1e9 / peak, "peak_source": peak_kind}


def fp64_rate(s, ms_per_step):
    """FP64 flop rate of the FP64 form: 12 transforms of 2.5 log2(Ngal1 Ngal2) flops per physical
    point (2.25 physical points per mode-point) + ~150 flops of solves per mode-point and
    substep, against the nominal FP64 rate of the part (1.25 TFLOP/s, not measured here)."""
    per_pt = 12 * 2.5 * math.log2(s.G1 * s.G2) * (s.G1 * s.G2) / (s.N1 * s.N2) + 150.0
    gf = per_pt * s.mode_points() * 3 / (ms_per_step * 1e-3) / 1e9
    return {"flops_per_mode_point": per_pt, "achieved_gflops": gf, "nominal_gflops": 1250.0,
            "frac_of_nominal": gf / 1250.0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="C1")
    ap.add_argument("--form", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--nonlin", default="products", choices=["products", "triads"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--error-steps", default="1,10,100",
                    help="mixed vs FP64 relative error after these step counts from the same start "
                         "(untimed, rank 0, both forms; 'none' to skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local, pg = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        barrier(pg)
        return

    import numpy as np
    import torch
    torch.cuda.set_device(local)
    from rnl_multiblock_nofft_gb300.native import GpuChannel
    from rnl_multiblock_nofft_gb300.workloads import initial_field, initial_scalars, workload_setup

    if args.workload == "C3":
        run_ensemble(args, ws, rank, pg, torch, np)
        barrier(pg)
        return
    s = workload_setup(args.workload)
    tl = triad_lists(args, s)
    mb = s.multiblock
    if mb:
        from rnl_multiblock_nofft_gb300.workloads import initial_field_bands
        icb = initial_field_bands(s, 1000 + rank)
        ic = [a for b in (1, 2, 3) for a in icb[b]]
    else:
        ic = initial_field(s, 1000 + rank)
    sc0 = initial_scalars(s)
    pts = s.mode_points()
    forms = ["fp64", "mixed"] if args.form == "both" else [args.form]
    res, states = {}, {}
    for form in forms:
        g = GpuChannel(s, form, triads=tl)
        if mb:
            g.upload_bands(icb)
        else:
            g.upload_state(*ic)
        g.set_scalars(**sc0)
        g.autotune()
        tuning = g.tuning()
        g.step(args.warmup)
        g.synchronize()
        barrier(pg)
        clk = ClockSampler(local)
        ms, launches = time_steps(g, args.steps, torch)
        clocks = clk.stop()
        barrier(pg)
        ms = reduce_max(pg, ms)
        res[form] = {"ms": ms, "launches": launches, "clocks": clocks, "tuning": tuning,
                     "value": ws * pts * 3 * args.steps / (ms * 1e-3) / 1e6}
        states[form] = ([a for b in (1, 2, 3) for a in g.download_bands()[b]] if mb else g.download_state())
        sc = g.scalars()
        res[form]["scalars"] = {k: sc[k] for k in ("t", "dt", "err", "Qx", "iter")}
        # per-kernel times (eager, events around each launch) for the roofline
        prof = g.profile_steps(1)
        res[form]["kernels"] = prof
        g.close()
        del g
        torch.cuda.empty_cache()

    # accuracy of the mixed form against the FP64 form after the same steps
    relerr = None
    if "fp64" in states and "mixed" in states:
        relerr = {}
        nf = 4
        for i, f in enumerate(("u1", "u2", "u3", "p")):
            a = np.concatenate([x.ravel() for x in states["fp64"][i::nf]])
            b = np.concatenate([x.ravel() for x in states["mixed"][i::nf]])
            relerr[f] = float(np.linalg.norm(b - a) / np.linalg.norm(a))
    vel_err = max(relerr[f] for f in ("u1", "u2", "u3")) if relerr else None
    head = "mixed" if ("mixed" in res and (relerr is None or vel_err <= 1e-5)) else "fp64"
    if "fp64" not in res:
        head = forms[0]
    R = res[head]

    peak, peak_kind = measured_peaks()
    for form, r in res.items():
        r["e2e"] = e2e_run(s, form, tl, ic, icb if mb else None, sc0, args.steps, ws, pg, torch, np)
        r["roofline"] = kernel_roofline(s, r["kernels"], form, tl, peak, peak_kind, args.workload)
        r["step_roofline"] = step_roofline(s, form, r["ms"] / args.steps, peak, peak_kind)
        if form == "fp64":
            r["fp64_rate"] = fp64_rate(s, r["ms"] / args.steps)
    line = {"metric": METRIC, "value": R["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": R["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "fp64" else "f32 transforms/products and Helmholtz solves; f64 state, (0,0) mode, pressure and flux correction",
            "data": "synthetic (seeded perturbed laminar channel, see rnl_multiblock_nofft_gb300/workloads.py)",
            "config": {"workload": f"{args.workload}: {workload_desc(args.workload)}", "form": head,
                       "mode_points_per_substep": pts, "N1": s.N1, "N2": s.N2, "ny": s.p.ny,
                       "core_band": [s.N1c, s.N2c] if mb else None,
                       "ny_with_immersed_region": s.nyv, "Ngal": [s.G1, s.G2],
                       "l2": "inputs larger than L2 (state ~%.0f MB)" % (sum(a.nbytes for a in ic) / 1e6),
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "roofline": R["roofline"], "step_roofline": R["step_roofline"], "gpu_launches": R["launches"],
            "clocks": R["clocks"], "e2e": R["e2e"],
            "forms": {f: {"value": r["value"], "ms_per_step": r["ms"] / args.steps, "scalars": r["scalars"],
                          "roofline": r["roofline"], "step_roofline": r["step_roofline"], "e2e": r["e2e"],
                          "autotuned": r["tuning"],
                          **({"fp64_rate": r["fp64_rate"]} if "fp64_rate" in r else {}),
                          "kernel_ms_per_step": {k: v[1] for k, v in r["kernels"].items()}}
                      for f, r in res.items()},
            "mixed_rel_err_vs_fp64": relerr}
    if tl is not None:
        nt = triad_terms(s, tl)
        tk = R["kernels"].get("k_triad")
        line["config"]["nonlinear"] = ("triad lists (ops_in_planes), complete (threshold 0): "
                                       f"{tl.n_triads() // max(1, len(tl.files))} triads per file")
        line["triads"] = {"complex_macs_per_substep": nt,
                          "k_triad_ms_per_step": tk[1] if tk else None,
                          "gflops": (8 * nt * 3 / (tk[1] * 1e-3) / 1e9) if tk else None}
    counts = [int(x) for x in args.error_steps.split(",") if x.strip().isdigit() and int(x) > 0]
    if rank == 0 and counts and "fp64" in res and "mixed" in res:
        line["mixed_rel_err_by_steps"] = error_by_steps(s, tl, icb if mb else ic, sc0, mb, counts)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s, triads=tl)
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(pg)


if __name__ == "__main__":
    main()
