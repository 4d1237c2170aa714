#!/usr/bin/env python
"""Benchmark: state-applies/s of the Γ-point wavefunction step (H psi + rho + ortho).

One step = rhoofr (density, kinetic energy and the reference's charge check)
+ vpsi + ortho(Gram-Schmidt) over all states of the cell, i.e. the three
hot-path routines a CPMD wavefunction-optimisation step calls
(forces_driver.mod.F90:165-224, updwf_utils.mod.F90:150).
state-applies/s = nstate * steps / time.

Workload: cubic L = 20.52 bohr, 64 atoms (2x2x2 diamond, +-0.05 bohr seeded
jitter), 128 states, 70 Ry (ngw = 42736), mesh 120^3; psi and V_loc seeded
synthetic.  The headline `value` is the mixed-precision path (FP32 FFT and
V*psi, FP64 accumulation, reductions and ortho); the plain FP64 drop-in is
measured in the same run (`fp64`).  Inputs (c0, c2: 87.5 MB each) are larger
than the 129 MB L2 together, so no L2 flush is needed between steps.

--impl reference times the reference's CPU path restated in C++/OpenMP FP64
(oracle/cpmd_port.cpp; the reference itself, Fortran + FFTW + BLAS, cannot be
built here): full 128-state steps on all host cores of rank 0.

Multi-GPU (torchrun): every rank runs an independent replica (the step does
not shard across GPUs in this build); value = total over ranks, time = max.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "state-applies/s (Hpsi+rho+ortho), mixed vs FP64 on same GB300 @|dE|<=1e-6 Ha/atom"
WORKLOAD = "cubic L=20.52 bohr, 64 atoms, 128 states, 70 Ry (ngw=42736), mesh 120^3, Gamma point"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """Clocks and throttle reasons sampled during the timed region: read through
    NVML (the driver's libnvidia-ml, read-only queries) every 2 ms, or nvidia-smi
    every 0.2 s where NVML cannot be loaded."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # NVML clocks-event reason bits: hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    BITS = (0x8, 0x40, 0x20, 0x4)

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.stop_ev = threading.Event()
        self.nvml = self._nvml()
        self.th = threading.Thread(target=self.run, daemon=True)

    def _nvml(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            for fn in ("nvmlDeviceGetClockInfo", "nvmlDeviceGetMaxClockInfo", "nvmlDeviceGetCurrentClocksEventReasons"):
                getattr(lib, fn)
            if lib.nvmlInit_v2() != 0:
                return None
            dev = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(dev)) != 0:
                return None
            return lib, dev
        except Exception:
            return None

    def _nvml_sample(self):
        import ctypes as C
        lib, dev = self.nvml
        sm, mx, reasons = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if lib.nvmlDeviceGetClockInfo(dev, 1, C.byref(sm)) != 0 or lib.nvmlDeviceGetMaxClockInfo(dev, 1, C.byref(mx)) != 0:
            return None
        if lib.nvmlDeviceGetCurrentClocksEventReasons(dev, C.byref(reasons)) != 0:
            return None
        r = reasons.value
        return [str(sm.value), str(mx.value), ""] + ["Active" if r & bit else "Not Active" for bit in self.BITS]

    def run(self):
        while not self.stop_ev.is_set():
            try:
                if self.nvml:
                    vals = self._nvml_sample()
                    if vals:
                        self.samples.append(vals)
                    self.stop_ev.wait(0.002)
                    continue
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                vals = [v.strip() for v in out.stdout.strip().split(",")]
                if len(vals) >= 7:
                    self.samples.append(vals)
            except Exception:
                pass
            self.stop_ev.wait(0.2)

    def __enter__(self):
        self.th.start()
        return self

    def __exit__(self, *a):
        self.stop_ev.set()
        self.th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples), "source": "nvml" if self.nvml else "nvidia-smi"}


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("GBCP_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- CPU reference (C++ port)
def bench_config(world: int) -> dict:
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD, "global_batch": 128 * world, "seq_len": 120 ** 3,
            "parallelism": "replicas" if world > 1 else "none",
            "l2": "inputs larger than L2 (c0+c2 = 175 MB)"}


def cpu_port_steps(cell, steps: int, warmup: int = 0, threads: int = 0, n_band=None):
    """Time the C++/OpenMP FP64 restatement of the step (rhoofr + vpsi + Gram-Schmidt)
    on the host cores.  n_band: time rhoofr + vpsi on the first n_band states only (a
    bounded sample of a large cell; then ortho is not timed).  Returns (seconds per step,
    threads, states the timed step covered)."""
    import numpy as np
    from oracle import cpmd_port as CP
    port = CP.Port(cell.basis, threads)
    c0 = np.asfortranarray(cell.c0 if n_band is None else cell.c0[:, :n_band])
    f = np.ascontiguousarray(cell.f[: c0.shape[1]])
    c2 = np.zeros_like(c0)
    work = c0.copy(order="F")

    def step():
        _, ek, cg, cr = port.rhoofr(work, f)
        if abs(cr - cg) > 1e-6:  # the reference's charge check (rhoofr_utils.mod.F90:625)
            raise RuntimeError("port: total density sums are not equal")
        port.vpsi(work, c2, f, cell.vpot)
        if n_band is None:
            port.rgs(work)

    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    t = (time.perf_counter() - t0) / max(1, steps)
    th = port.threads
    port.close()
    return t, th, c0.shape[1]


def run_reference(args, rank, world):
    """The reference arm: the C++/OpenMP FP64 restatement of rhoofr + vpsi + rgs
    (the reference's own Fortran/FFTW/BLAS build is not possible here), full
    128-state steps of the 64-atom cell on all host cores of rank 0."""
    if rank != 0:
        return
    from cpmd_gb300.synth import make_cell
    cell = make_cell("c1")
    t, th, _ = cpu_port_steps(cell, args.steps, args.warmup)
    value = cell.nstate / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "state-applies/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded psi, V_loc)",
        "config": bench_config(world),
        "cpu_baseline": {"value": value, "unit": "state-applies/s", "cores": th, "kind": "port",
                         "sample": f"C++/OpenMP FP64 restatement of rhoofr + vpsi + Gram-Schmidt ortho "
                                   f"(oracle/cpmd_port.cpp), full {cell.nstate}-state steps, {th} threads"},
        "e2e": {"value": value, "unit": "state-applies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# mixed config-1 kernels (64 pairs per launch), from one ncu capture of this
# script's own command (python bench.py --steps 2 --warmup 3 --fp64-steps 1
# --e2e-steps 1 --no-cpu --no-extras; k_xrho_fs: -k regex:k_xrho_fs -s 2 -c 1):
# the density x-stage, and the three-stage vpsi x-stage used with plane = 0.
NCU_TRAFFIC = {"k_xinv_rho": 419.589632e6 + 31.977216e6, "k_xvx": 412.769536e6 + 348.129792e6}


def kernel_bytes(name: str, geo: dict, np_: int, s: int) -> float:
    """Compulsory HBM bytes of one launch (s = bytes per complex of the FFT precision)."""
    n1, n2, n3 = geo["nr"]
    ncol, nslot, nent, ngw = geo["ncol"], geo["nslot"], geo["nent"], geo["ngw"]
    zb = n3 * ncol * s
    yb = n3 * n2 * nslot * s
    grid = n1 * n2 * n3
    if name == "k_zinv":
        return np_ * (2 * ngw * 16 + zb)
    if name == "k_wfn_sum":  # the states' checksum of the kept Z stage: one read of c0
        return np_ * 2 * ngw * 16
    if name == "k_yinv":
        return np_ * (zb + yb)
    if name == "k_xinv_rho":
        return np_ * yb + 2 * grid * 8
    if name == "k_xvx":
        return np_ * 2 * yb + grid * (s // 2)      # V(r) in the transform precision
    if name == "k_yfwd":
        return np_ * (yb + zb)
    if name == "k_zfwd":
        return np_ * (zb + nent * s)
    if name == "k_decode":
        return np_ * (2 * ngw * s + 2 * ngw * 16 + 2 * 2 * ngw * 16)
    if name == "k_plane_rho":                       # zbuf read, rho read + write
        return np_ * zb + 2 * grid * 8
    if name == "k_plane_vx":                        # zbuf read and written in place, V(r) in FP32
        return 2 * np_ * zb + grid * 4
    return 0.0


def kernel_fft_flops(name: str, geo: dict, np_: int) -> float:
    """Algorithmic FP32 FLOPs of one launch of the plane-fused kernels (5 N log2 N per
    complex line transform: the slot lines in y and the rows in x of every z-plane)."""
    import math
    n1, n2, n3 = geo["nr"]
    nslot = geo["nslot"]
    line = 5.0 * n1 * math.log2(n1)
    per_plane = line * (nslot + n2)
    if name == "k_plane_rho":
        return np_ * n3 * (per_plane + 4.0 * n1 * n2)
    if name == "k_plane_vx":
        return np_ * n3 * (2.0 * per_plane + 2.0 * n1 * n2)
    return 0.0


def fp32_peak_tflops() -> float:
    """FP32 FMA peak of the SIMT pipes: 152 SMs x 128 lanes x 2 FLOPs at the maximum SM
    clock of MEASURED_PEAKS.json (nominal; the copy and GEMM peaks there are measured)."""
    mhz = 2070.0
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        mhz = float(json.loads(p.read_text()).get("sm_max_mhz", mhz))
    return 152 * 128 * 2 * mhz * 1e6 / 1e12


def kernel_flops(name: str, n: int, ngw: int) -> float:
    """bf16 tensor-core FLOPs one launch of the split-precision ortho GEMMs issues:
    36 digit-pair products per 128 x 64 output tile, K = 2 ngw (S) or the
    triangular extent of U^-1 (C U^-1)."""
    K = 2 * ngw
    mt, nt = -(-n // 128), -(-n // 64)
    if name == "k_ozaki_syrk":
        tiles = sum(max(0, nt - 2 * ib) for ib in range(mt))
        return tiles * 128 * 64 * K * 2 * 36
    if name == "k_ozaki_rmul":
        rt = -(-K // 128)
        return sum(rt * 128 * 64 * min(n, 64 * (j + 1)) * 2 * 36 for j in range(nt))
    return 0.0


def run_gpu(args, rank, world, local):
    import numpy as np
    import torch
    from cpmd_gb300 import Context, kernel_launches
    from cpmd_gb300.synth import make_cell

    torch.cuda.set_device(local)
    cell = make_cell("c1")
    b = cell.basis
    n = cell.nstate
    dev = torch.device("cuda", local)
    c0 = torch.from_numpy(np.ascontiguousarray(cell.c0.T)).to(dev)
    f = torch.from_numpy(cell.f).to(dev)
    v = torch.from_numpy(cell.vpot).to(dev)
    rho = torch.empty(tuple(b.kr[::-1]), dtype=torch.float64, device=dev)
    c2 = torch.zeros_like(c0)

    def make_step(ctx):
        # the reference's full rhoofr: density, kinetic energy and the charge check
        # (the library returns an error when |csumr - csumg| fails it)
        def step():
            ctx.rhoofr(c0, f, rho, energies=True)
            ctx.vpsi(c0, c2, f, v)
            ctx.ortho(c0, "gs")
        return step

    def timed(ctx, steps, warmup, sample_clocks=False):
        step = make_step(ctx)
        for _ in range(warmup):
            step()
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        l0 = kernel_launches()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.__enter__()
        s.record()
        for _ in range(steps):
            step()
        e.record()
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
        barrier(world)
        ms = s.elapsed_time(e)
        return ms, kernel_launches() - l0, (sampler.summary() if sampler else None)

    batch = args.batch
    ctx_mx = Context(b, "mixed", batch=batch)
    ctx_64 = Context(b, "fp64", batch=batch)
    ms_mx, launches, clocks = timed(ctx_mx, args.steps, args.warmup, sample_clocks=True)
    ms_mx = allreduce_max(ms_mx, world)
    ms_64, _, _ = timed(ctx_64, args.fp64_steps, max(1, min(args.warmup, 2)))
    ms_64 = allreduce_max(ms_64, world)

    value = world * n * args.steps / (ms_mx / 1e3)
    v64 = world * n * args.fp64_steps / (ms_64 / 1e3)

    # accuracy of the mixed step against FP64 on the same inputs: energy E_kin + int V rho
    rho64, ek64, _, _ = ctx_64.rhoofr(c0, f)
    rhomx, ekmx, _, _ = ctx_mx.rhoofr(c0, f)
    dv = b.omega / (b.nr[0] * b.nr[1] * b.nr[2])
    e64 = ek64 + dv * float((rho64 * v).sum())
    emx = ekmx + dv * float((rhomx * v).sum())
    nat = cell.tau.shape[0]

    # live per-kernel timing (CUDA events on the library stream) over profiled steps
    ctx_mx.profile(True)
    for _ in range(2):
        make_step(ctx_mx)()
    prof = ctx_mx.profile_read()
    ctx_mx.profile(False)
    geo = geometry_summary(b)
    npairs = (n + 1) // 2
    bt = min(batch, npairs)
    # the roofline line: the dominant kernel by time among those bound by HBM bandwidth
    # (the FFT stages with an HBM byte model and the split GEMMs); the plane-fused FFT
    # kernels are FP32-issue bound and are reported against the FP32 pipe in `stages`
    cand = {k: v for k, v in prof.items()
            if kernel_flops(k, n, b.ngw) or (kernel_bytes(k, geo, bt, 8) and not kernel_fft_flops(k, geo, 1))}
    dom = max((cand or prof).items(), key=lambda kv: kv[1][0])
    dname, (dms, dcount) = dom
    hbm, bf16, src = peaks()
    per_launch_ms = dms / dcount
    bytes_per_launch = kernel_bytes(dname, geo, bt, 8)
    flops_per_launch = kernel_flops(dname, n, b.ngw)
    if flops_per_launch:
        bound, unit, peak, work = "tensor", "TFLOP/s", bf16, flops_per_launch
        achieved = flops_per_launch / (per_launch_ms / 1e3) / 1e12
    else:
        bound, unit, peak, work = "hbm", "GB/s", hbm, bytes_per_launch
        achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9 if bytes_per_launch else None
    step_ms_prof = sum(t for t, _ in prof.values()) / 2

    # end to end through the public API with host (pinned) buffers
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    c0h = pin((n, b.ngw), torch.complex128)
    c0h[:] = cell.c0.T
    c0h = c0h.T  # Fortran (ngw, n) view of pinned memory
    c2h = pin((n, b.ngw), torch.complex128)
    c2h[:] = 0
    c2h = c2h.T
    fh = pin((n,), torch.float64)
    fh[:] = cell.f
    vh = pin(tuple(b.kr[::-1]), torch.float64)
    vh[:] = cell.vpot
    rhoh = pin(tuple(b.kr[::-1]), torch.float64)

    calls = {"rhoofr": 0.0, "vpsi": 0.0, "ortho": 0.0}

    def e2e_run(ctx, steps, split=None):
        def e2e_step():
            t = time.perf_counter()
            ctx.rhoofr(c0h, fh, rhoh, energies=True)
            t1 = time.perf_counter()
            ctx.vpsi(c0h, c2h, fh, vh)
            t2 = time.perf_counter()
            ctx.ortho(c0h, "gs")
            t3 = time.perf_counter()
            return t1 - t, t2 - t1, t3 - t2
        for _ in range(2):
            e2e_step()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            r = e2e_step()
            if split is not None:
                for k, v in zip(("rhoofr", "vpsi", "ortho"), r):
                    split[k] += v / steps
        return allreduce_max(time.perf_counter() - t0, world)

    # rhoofr's upload of c0 serves vpsi and ortho as well (the reference's cp_cuwfn cache)
    ctx_mx.set_option("wfn_cache", 1)
    t_e2e = e2e_run(ctx_mx, args.e2e_steps, calls)
    c0h[:] = cell.c0
    t_e2e64 = e2e_run(ctx_64, 2)
    wfn = b.ngw * n * 16
    grid = b.nnr1 * 8
    h2d = wfn + wfn + 2 * n * 8 + grid        # c0 (rhoofr), c2 (vpsi), f twice, V(r)
    d2h = grid + wfn + wfn                    # rho, c2, the orthonormalised c0
    e2e = world * n * args.e2e_steps / t_e2e
    e2e64 = world * n * 2 / t_e2e64

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        t_cpu, th, _ = cpu_port_steps(cell, 2, 1)
        cpu = {"value": n / t_cpu, "unit": "state-applies/s", "cores": th, "kind": "port",
               "sample": f"C++/OpenMP FP64 restatement (oracle/cpmd_port.cpp) of rhoofr + vpsi + Gram-Schmidt, "
                         f"2 full {n}-state steps after 1 warm-up, {th} threads"}

    extras = None
    if rank == 0 and world == 1 and not args.no_extras:
        del c0h, c2h
        extras = run_extras(args, dev)

    # every band-loop stage against the HBM roof (algorithmic bytes per launch / mean launch time)
    fp32_peak = fp32_peak_tflops()
    stages = {}
    for k, (t_ms, cnt) in prof.items():
        by = kernel_bytes(k, geo, bt, 8)
        if by and cnt:
            gbs = by / (t_ms / cnt / 1e3) / 1e9
            stages[k] = {"ms_per_step": round(t_ms / 2, 4), "GB_s": round(gbs, 1), "frac": round(gbs / hbm, 3)}
            fl = kernel_fft_flops(k, geo, bt)
            if fl:
                tf = fl / (t_ms / cnt / 1e3) / 1e12
                stages[k].update({"fp32_tflops": round(tf, 2), "frac_fp32": round(tf / fp32_peak, 3),
                                  "fp32_peak": round(fp32_peak, 1)})

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "state-applies/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mx / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-fft/f64-accum", "data": "synthetic (seeded psi, V_loc)",
            "config": bench_config(world),
            "run": {"precision": "mixed", "pairs_per_batch": bt, "step": "rhoofr (with E_kin and the charge check) "
                    "+ vpsi + Gram-Schmidt ortho over all 128 states"},
            "fp64": {"value": v64, "ms_per_step": ms_64 / args.fp64_steps, "steps": args.fp64_steps,
                     "mixed_over_fp64": value / v64},
            "accuracy": {"dE_Ha_per_atom_mixed_vs_fp64": abs(emx - e64) / nat, "E_fp64_Ha": e64},
            "roofline": {"bound": bound, "kernel": dname, "achieved": achieved, "peak": peak, "unit": unit,
                         "frac": (achieved / peak) if achieved else None, "traffic": NCU_TRAFFIC.get(dname),
                         "peak_source": src, "launch_ms": per_launch_ms, "work_per_launch": work,
                         "kernel_share": dms / 2 / step_ms_prof, "stages": stages},
            "kernels_ms_per_step": {k: round(t / 2, 4) for k, (t, _) in sorted(prof.items(), key=lambda kv: -kv[1][0])},
            "clocks": clocks,
            "e2e": {"value": e2e, "unit": "state-applies/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": args.e2e_steps,
                    "ms_per_call": {k: round(v * 1e3, 4) for k, v in calls.items()}, "path": "C ABI, host (pinned) buffers, GBCP_MEM_HOST; c0 uploaded once "
                                                      "per step by rhoofr and reused by vpsi and ortho "
                                                      "(GBCP_OPT_WFN_CACHE)",
                    "fp64_drop_in": {"value": v64, "e2e_value": e2e64, "ms_per_step": ms_64 / args.fp64_steps,
                                     "mixed_over_fp64": value / v64,
                                     "note": "the plain FP64 drop-in on the same cell, device-resident "
                                             "(value) and through host buffers (e2e_value)"}},
            "gpu_launches": launches,
            "cpu_baseline": cpu,
            "other_configs": extras,
        }
        print(json.dumps(line), flush=True)
    ctx_mx.close()
    ctx_64.close()


def cpu_band_sample(cl, n_band: int) -> dict:
    """CPU baseline of a large device-resident cell: the C++/OpenMP FP64
    restatement's rhoofr + vpsi on its first n_band states (copied to the host),
    one timed call after one warm-up; the rate is per state of the band loop
    only (the rest of the cell's step is not in the sample)."""
    import types
    import numpy as np
    c0 = np.asfortranarray(cl.c0[:n_band].cpu().numpy().T)
    host = types.SimpleNamespace(basis=cl.basis, c0=c0, f=cl.f[:n_band].cpu().numpy(),
                                 vpot=np.ascontiguousarray(cl.vpot.cpu().numpy()))
    t, th, ns = cpu_port_steps(host, 1, 1, n_band=n_band)
    return {"value": ns / t, "unit": "state-applies/s (band loop only)", "cores": th, "kind": "port",
            "sample": f"C++/OpenMP FP64 restatement: rhoofr + vpsi on {ns} of {cl.nstate} states, one call after "
                      f"one warm-up, {th} threads; ortho, projectors and the energy terms not timed"}


def _timed_loop(step, steps, warmup):
    import torch
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        step()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / steps


def run_extras(args, dev):
    """The other cells of the hot path, one GPU, inputs resident on the device:
    the 8-atom cell (16 states, 32^3), the energy + adjoint of the 216-atom cell
    (432 states, 144^3) and the 512-atom projector/Loewdin cell (1024 states,
    240^3, 4096 projectors).  Each is timed with CUDA events after warm-up."""
    import numpy as np
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.synth import gaussian_form_factor, make_cell, make_cell_device

    out = {}
    # ---- 8 atoms, 16 states, 32^3, GS ortho
    cl = make_cell("c0")
    b = cl.basis
    c0 = torch.from_numpy(np.ascontiguousarray(cl.c0.T)).to(dev)
    f = torch.from_numpy(cl.f).to(dev)
    v = torch.from_numpy(cl.vpot).to(dev)
    rho = torch.empty(tuple(b.kr[::-1]), dtype=torch.float64, device=dev)
    c2 = torch.zeros_like(c0)
    r = {}
    for prec in ("mixed", "fp64"):
        ctx = Context(b, prec)

        def step():
            ctx.rhoofr(c0, f, rho, energies=True)
            ctx.vpsi(c0, c2, f, v)
            ctx.ortho(c0, "gs")
        ms = _timed_loop(step, 50, 5)
        r[prec] = {"state_applies_per_s": cl.nstate / (ms / 1e3), "ms_per_step": ms}
        ctx.close()
    t_cpu, th, _ = cpu_port_steps(cl, 20, 2)
    r["cpu_baseline"] = {"value": cl.nstate / t_cpu, "unit": "state-applies/s", "cores": th, "kind": "port",
                         "sample": "C++/OpenMP FP64 restatement, 20 full 16-state steps (rhoofr + vpsi + rgs)"}
    out["cell_8atoms_16states_32cubed"] = r

    # ---- CP-dynamics constraint (rortog) on the 64-atom cell: 128 states, ngw 42 736
    cl = make_cell_device("c1")
    b = cl.basis
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)
    noise = torch.complex(torch.randn(cl.c0.shape, generator=gen, device=dev, dtype=torch.float64),
                          torch.randn(cl.c0.shape, generator=gen, device=dev, dtype=torch.float64))
    cm0 = cl.c0 + 1e-3 * noise / float(np.sqrt(b.ngw))
    if b.geq0:
        cm0[:, 0] = cm0[:, 0].real.to(torch.complex128)
    cm = torch.empty_like(cm0)
    r = {}
    gams = {}
    for prec in ("mixed", "fp64"):
        ctx = Context(b, prec)
        holder = {}

        def step():
            cm.copy_(cm0)
            holder["g"], holder["it"] = ctx.rortog(cl.c0, cm, epsog=1e-6, maxit=30)
        ms = _timed_loop(step, 5 if prec == "mixed" else 2, 2)
        gams[prec] = holder["g"].clone()
        s = ctx.ovlap(cm)
        r[prec] = {"ms_per_call": ms, "iterations": holder["it"],
                   "max_abs_overlap_minus_identity_after": float((s - torch.eye(cl.nstate, device=dev,
                                                                                dtype=torch.float64)).abs().max())}
        ctx.close()
    r["max_abs_gam_mixed_vs_fp64"] = float((gams["mixed"] - gams["fp64"]).abs().max())
    r["workload"] = ("rortog (rortho iteration + cm += c0 gam), 128 states, ngw 42736, cm = c0 + 1e-3 noise, "
                     "epsog 1e-6; each call includes an 87.5 MB device copy restoring cm")
    out["rortog_64atoms_128states"] = r
    del cl, cm, cm0, noise, gams
    torch.cuda.empty_cache()

    # ---- 216 atoms, 432 states, 50 Ry, 144^3: energy + adjoint (dE/dpsi*, dE/dV, forces)
    cl = make_cell_device("c2")
    b = cl.basis
    vps = torch.from_numpy(gaussian_form_factor(b)).to(dev)
    tau = torch.from_numpy(cl.tau).to(dev)
    isp = np.zeros(len(cl.tau), dtype=np.int32)
    r = {}
    res = {}
    for prec in ("mixed", "fp64"):
        ctx = Context(b, prec)
        holder = {}

        def step():
            holder["r"] = ctx.energy(cl.c0, cl.f, tau, vps, isp)
        ms = _timed_loop(step, 3 if prec == "mixed" else 2, 2 if prec == "mixed" else 1)
        res[prec] = holder["r"]
        r[prec] = {"state_applies_per_s": cl.nstate / (ms / 1e3), "ms_per_energy_and_gradient": ms}
        ctx.close()
    nat = len(cl.tau)
    r["dE_Ha_per_atom_mixed_vs_fp64"] = abs(res["mixed"][0]["etot"] - res["fp64"][0]["etot"]) / nat
    r["dF_max_Ha_per_bohr_mixed_vs_fp64"] = float((res["mixed"][3] - res["fp64"][3]).abs().max())
    r["E_fp64_Ha"] = res["fp64"][0]["etot"]
    r["workload"] = "E = kinetic + local + Hartree + LDA-PZ and its adjoint, 216 atoms, 432 states, 50 Ry, 144^3"
    # the same with the gradient-corrected functional (PBE): + 7 dense FFTs of 144^3 per call
    pbe = {}
    for prec in ("mixed", "fp64"):
        ctx = Context(b, prec)
        ctx.set_option("xc", 1)
        holder = {}

        def step():
            holder["r"] = ctx.energy(cl.c0, cl.f, tau, vps, isp)
        ms = _timed_loop(step, 3 if prec == "mixed" else 2, 2 if prec == "mixed" else 1)
        pbe[prec] = {"ms_per_energy_and_gradient": ms, "E_Ha": holder["r"][0]["etot"],
                     "F": holder["r"][3]}
        ctx.close()
    r["pbe"] = {"mixed_ms_per_energy_and_gradient": pbe["mixed"]["ms_per_energy_and_gradient"],
                "fp64_ms_per_energy_and_gradient": pbe["fp64"]["ms_per_energy_and_gradient"],
                "dE_Ha_per_atom_mixed_vs_fp64": abs(pbe["mixed"]["E_Ha"] - pbe["fp64"]["E_Ha"]) / nat,
                "dF_max_Ha_per_bohr_mixed_vs_fp64": float((pbe["mixed"]["F"] - pbe["fp64"]["F"]).abs().max()),
                "E_fp64_Ha": pbe["fp64"]["E_Ha"]}
    r["cpu_baseline"] = cpu_band_sample(cl, 16)
    out["adjoint_216atoms_432states_144cubed"] = r
    del cl, res, holder, vps, tau
    torch.cuda.empty_cache()

    # ---- 512 atoms, 1024 states, 70 Ry, 240^3, 4096 projectors, Loewdin
    cl = make_cell_device("c4")
    b = cl.basis
    p = cl.proj
    nat = len(cl.tau)
    rho = torch.empty(tuple(b.kr[::-1]), dtype=torch.float64, device=dev)
    fnl = torch.empty((cl.nstate, 8, nat), dtype=torch.float64, device=dev)
    r = {}
    energies = {}
    dv = b.omega / (b.nr[0] * b.nr[1] * b.nr[2])
    for prec in ("mixed", "fp64"):
        ctx = Context(b, prec)
        c = cl.c0.clone()
        c2 = torch.zeros_like(c)

        def step():
            ctx.rhoofr(c, cl.f, rho, energies=True)
            ctx.vpsi(c, c2, cl.f, cl.vpot)
            ctx.rnlsm(c, p["twnl"], p["eigr"], p["nghtol"], fnl)
            ctx.fnonloc(c2, cl.f, fnl, p["twnl"], p["eigr"], p["nghtol"], p["wsg"])
            ctx.ortho(c, "lowdin")
        ms = _timed_loop(step, 3 if prec == "mixed" else 1, 2 if prec == "mixed" else 1)
        if prec == "mixed":
            # per-kernel CUDA-event times of one step; the tensor-core GEMMs against the sustained peak
            ctx.profile(True)
            step()
            kp = ctx.profile_read()
            ctx.profile(False)
        rh, ek, _, _ = ctx.rhoofr(c, cl.f, rho)
        energies[prec] = ek + dv * float((rh * cl.vpot).sum())
        scond = ctx.ortho(c, "lowdin")          # max|S - I| of the orthonormalised states
        r[prec] = {"state_applies_per_s": cl.nstate / (ms / 1e3), "ms_per_step": ms,
                   "orthonormality_after_ortho": scond}
        if prec == "mixed":
            r[prec]["kernels_ms_per_step"] = {k: round(t, 3) for k, (t, _) in
                                              sorted(kp.items(), key=lambda kv: -kv[1][0])[:14]}
            P = 8 * nat
            K = 2 * b.ngw
            # rnlsm1 + fnonloc: 2 x (2 P n K) FLOPs of the FP32-class product, 6 bf16 slice pairs each
            proj = 2 * 2.0 * P * cl.nstate * K
            if "k_tc_gemm" in kp:
                t_tc = kp["k_tc_gemm"][0] / 1e3
                r[prec]["projector_gemms"] = {
                    "ms": kp["k_tc_gemm"][0], "fp32_class_tflops": proj / t_tc / 1e12,
                    "bf16_issued_tflops": 6 * proj / t_tc / 1e12,
                    "frac_of_sustained_bf16": 6 * proj / t_tc / 1e12 / float(json.loads(
                        (ROOT / "MEASURED_PEAKS.json").read_text()).get("bf16_tflops_sustained", 1714.6))
                    if (ROOT / "MEASURED_PEAKS.json").exists() else None}
            if "k_ozaki_ns" in kp:
                tns, cnt = kp["k_ozaki_ns"]
                # each n x n x n split product issues 36 digit-pair bf16 MMAs per 128 x 32 output tile and K step
                ns_flops = cnt * 2.0 * cl.nstate ** 3 * 36
                r[prec]["loewdin_ns_gemms"] = {"ms": tns, "products": cnt,
                                               "bf16_issued_tflops": ns_flops / (tns / 1e3) / 1e12}
            # non-local forces of the same states: rnlsm2 (3 x 4096 derivative projectors) + rnlfor
            dfnl = torch.empty((cl.nstate, 3, 8, nat), dtype=torch.float64, device=dev)
            fion = torch.zeros((nat, 3), dtype=torch.float64, device=dev)

            def forces():
                ctx.rnlsm(c, p["twnl"], p["eigr"], p["nghtol"], fnl)
                ctx.rnlsm2(c, p["twnl"], p["eigr"], p["nghtol"], dfnl)
                ctx.rnlfor(cl.f, fnl, dfnl, p["wsg"], fion)
            r[prec]["nl_forces_ms"] = _timed_loop(forces, 2, 1)
            del dfnl, fion
        del c, c2
        ctx.close()
        torch.cuda.empty_cache()
    r["dE_Ha_per_atom_mixed_vs_fp64"] = abs(energies["mixed"] - energies["fp64"]) / nat
    r["workload"] = ("rhoofr + vpsi + rnlsm1 + fnonloc + Loewdin ortho, 512 atoms, 1024 states, 70 Ry "
                     f"(ngw={b.ngw}), 240^3, 4096 projectors; nl_forces_ms = rnlsm1 + rnlsm2 + rnlfor")
    r["cpu_baseline"] = cpu_band_sample(cl, 16)
    out["projectors_512atoms_1024states_240cubed"] = r
    del cl, p, rho, fnl
    torch.cuda.empty_cache()

    # ---- 64 independent cells (8/16/32/64 atoms, 16-128 states, 30 Ry, 36^3-72^3), one graph launch per step
    from cpmd_gb300 import Batch
    from cpmd_gb300.synth import make_batch
    cells = make_batch(64)
    nst = sum(cc.c0.shape[1] for cc in cells)

    def io_of(c64=False):
        io = []
        dt = torch.complex64 if c64 else torch.complex128
        for cc in cells:
            bb = cc.basis
            io.append(dict(c0=torch.from_numpy(np.ascontiguousarray(cc.c0.T)).to(dev).to(dt),
                           f=torch.from_numpy(cc.f).to(dev), vpot=torch.from_numpy(cc.vpot).to(dev),
                           rhoe=torch.empty(tuple(bb.kr[::-1]), dtype=torch.float64, device=dev),
                           c2=torch.zeros((cc.c0.shape[1], bb.ngw), dtype=dt, device=dev)))
        return io

    r = {}
    en = {}
    # the configuration as specified (complex64 states, FP64 energies), then complex128
    # states in the mixed and FP64 precisions
    for key, prec, c64 in (("mixed_c64", "mixed", True), ("mixed", "mixed", False), ("fp64", "fp64", False)):
        io = io_of(c64)
        bt = Batch([cc.basis for cc in cells], prec, nstreams=len(cells))
        report = bt.tune(io)
        en[key] = bt.step(io)[0]
        for _ in range(3):
            bt.step(io)
        steps = 10
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            bt.step(io)
        ms = (time.perf_counter() - t0) / steps * 1e3
        r[key] = {"state_applies_per_s": nst / (ms / 1e3), "ms_per_step": ms, "states": "complex64" if c64 else
                  "complex128", "kernels_per_graph_launch": bt.graph_kernels(),
                  "autotuner": report.strip().split("\n")}
        if c64:
            # orthonormality of the stored complex64 states after the last step's ortho
            worst = 0.0
            for cc, x in zip(cells, io):
                cm = x["c0"].to(torch.complex128)
                sm = 2.0 * (cm.conj() @ cm.T).real
                if cc.basis.geq0:
                    sm -= torch.outer(cm[:, 0].real, cm[:, 0].real)
                worst = max(worst, float((sm - torch.eye(sm.shape[0], dtype=sm.dtype, device=dev)).abs().max()))
            r[key]["orthonormality_after_ortho"] = worst
        bt.close()
        del io
    # the same cells through one context each, no graph, one stream
    io = io_of()
    ctxs = [Context(cc.basis, "mixed") for cc in cells]

    def seq():
        for cx_, x in zip(ctxs, io):
            cx_.rhoofr(x["c0"], x["f"], x["rhoe"], energies=True)
            cx_.vpsi(x["c0"], x["c2"], x["f"], x["vpot"])
            cx_.ortho(x["c0"], "gs")
        torch.cuda.synchronize()
    seq()
    t0 = time.perf_counter()
    for _ in range(3):
        seq()
    ms_seq = (time.perf_counter() - t0) / 3 * 1e3
    for cx_ in ctxs:
        cx_.close()
    nats = np.array([cc.tau.shape[0] for cc in cells])
    de = np.abs(en["mixed"].sum(axis=1) - en["fp64"].sum(axis=1)) / nats
    de64 = np.abs(en["mixed_c64"].sum(axis=1) - en["fp64"].sum(axis=1)) / nats
    r["mixed_sequential_contexts"] = {"state_applies_per_s": nst / (ms_seq / 1e3), "ms_per_step": ms_seq}
    r["dE_Ha_per_atom_mixed_vs_fp64_max"] = float(de.max())
    r["dE_Ha_per_atom_mixed_c64_vs_fp64_max"] = float(de64.max())
    # CPU baseline: the C++/OpenMP restatement on one cell of each size class (full steps),
    # weighted by the number of cells in the class
    classes = {}
    for cc in cells:
        classes.setdefault((tuple(cc.basis.nr), cc.basis.ngw, cc.c0.shape[1]), []).append(cc)
    t_all, th = 0.0, 1
    for members in classes.values():
        t, th, _ = cpu_port_steps(members[0], 2, 1)
        t_all += t * len(members)
    r["cpu_baseline"] = {"value": nst / t_all, "unit": "state-applies/s", "cores": th, "kind": "port",
                         "sample": f"C++/OpenMP FP64 restatement, 2 full steps of one cell per size class "
                                   f"({len(classes)} classes) scaled by the class counts, {th} threads"}
    r["timing"] = "host wall clock per step: one cudaGraphLaunch + stream synchronise"
    r["workload"] = (f"64 cells, atoms uniform in {{8,16,32,64}}, {nst} states in total, 30 Ry, meshes 36^3-72^3, "
                     "rhoofr + vpsi + GS ortho")
    out["batch_64cells"] = r
    return out


def run_case_projectors(args):
    """Mixed-precision projector contractions (rnlsm1 + fnonloc on the tensor
    cores) on a mid-size synthetic problem: the 64-atom cell's sphere
    (ngw = 42.7k), 128 atoms x 8 projectors, 512 states.  Small enough
    (about 2 GB on the device) for a profiler to replay."""
    import numpy as np
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.cell import make_basis

    b = make_basis(20.52, 120, 70.0)
    n, nat, ngh = args.case_states, args.case_atoms, 8
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    c0 = torch.complex(torch.randn(n, b.ngw, generator=g, device="cuda", dtype=torch.float64),
                       torch.randn(n, b.ngw, generator=g, device="cuda", dtype=torch.float64)) * 0.01
    tw = torch.rand(ngh, b.ngw, generator=g, device="cuda", dtype=torch.float64)
    eig = torch.exp(1j * 6.283185307179586 * torch.rand(nat, b.ngw, generator=g, device="cuda", dtype=torch.float64))
    nghtol = np.array([0, 1, 1, 1, 0, 1, 1, 1], dtype=np.int32)
    f = torch.full((n,), 2.0, dtype=torch.float64, device="cuda")
    wsg = torch.rand(ngh, generator=g, device="cuda", dtype=torch.float64)
    fnl = torch.empty((n, ngh, nat), dtype=torch.float64, device="cuda")
    c2 = torch.zeros_like(c0)
    ctx = Context(b, "mixed")

    def step():
        ctx.rnlsm(c0, tw, eig, nghtol, fnl)
        ctx.fnonloc(c2, f, fnl, tw, eig, nghtol, wsg)
    ms = _timed_loop(step, args.steps, args.warmup)
    flop = 2 * 2.0 * nat * ngh * n * 2 * b.ngw      # both GEMMs, FP32-equivalent
    print(json.dumps({"case": "projectors", "ms_per_pair_of_calls": ms, "states": n, "projectors": nat * ngh,
                      "ngw": b.ngw, "tflops_fp32_equivalent": flop / (ms / 1e3) / 1e12,
                      "tflops_bf16_issued": 6 * flop / (ms / 1e3) / 1e12}), flush=True)
    ctx.close()


def run_case_loewdin(args):
    """Loewdin ortho of --case-states states (1024 by default for this case) on the
    64-atom cell's sphere (ngw = 42.7k): the overlap GEMM (K = 85 472) and the
    Newton-Schulz products S^-1/2 (n x n x n) on the tensor cores, FP64-accurate.
    About 2 GB on the device."""
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.cell import make_basis

    b = make_basis(20.52, 120, 70.0)
    n = args.case_states if args.case_states != 512 else 1024
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    c0 = torch.complex(torch.randn(n, b.ngw, generator=g, device="cuda", dtype=torch.float64),
                       torch.randn(n, b.ngw, generator=g, device="cuda", dtype=torch.float64)) * 0.01
    ctx = Context(b, "mixed")
    work = torch.empty_like(c0)

    def step():
        work.copy_(c0)
        ctx.ortho(work, "lowdin")
    ms = _timed_loop(step, args.steps, args.warmup)
    ctx.profile(True)
    step()
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    ns_ms, ns_n = prof.get("k_ozaki_ns", (0.0, 0))
    # every Newton-Schulz product is an n x n x n product of 36 bf16 digit pairs (s + t <= 7)
    ns_tflops = 36 * 2.0 * n ** 3 * ns_n / (ns_ms / 1e3) / 1e12 if ns_ms else None
    print(json.dumps({"case": "loewdin", "ms_per_ortho": ms, "states": n, "ngw": b.ngw,
                      "ns_products": ns_n, "ns_ms": ns_ms, "ns_bf16_issued_tflops": ns_tflops,
                      "kernels_ms": {k: round(v[0], 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}}),
          flush=True)
    ctx.close()


def run_case_timeline(args):
    """One config-1 step through the C ABI with pinned host buffers (rhoofr, vpsi,
    Gram-Schmidt ortho; the wavefunction cache on), after 5 warm-up steps, with the
    library's per-launch event timers: one JSON line per kernel or copy (name, lane:
    0 kernels, 1 uploads, 2 downloads; start and end in ms from the first record).
    The timers add a few microseconds per launch."""
    import torch
    from cpmd_gb300 import Context
    from cpmd_gb300.synth import make_cell
    cell = make_cell("c1")
    b, n = cell.basis, cell.nstate
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()  # noqa: E731
    c0h = pin((n, b.ngw), torch.complex128)
    c0h[:] = cell.c0.T
    c0h = c0h.T
    c2h = pin((n, b.ngw), torch.complex128)
    c2h[:] = 0
    c2h = c2h.T
    fh = pin((n,), torch.float64)
    fh[:] = cell.f
    vh = pin(tuple(b.kr[::-1]), torch.float64)
    vh[:] = cell.vpot
    rhoh = pin(tuple(b.kr[::-1]), torch.float64)
    ctx = Context(b, "mixed")
    ctx.set_option("wfn_cache", 1)

    def step():
        t = [time.perf_counter()]
        ctx.rhoofr(c0h, fh, rhoh, energies=True)
        t.append(time.perf_counter())
        ctx.vpsi(c0h, c2h, fh, vh)
        t.append(time.perf_counter())
        ctx.ortho(c0h, "gs")
        t.append(time.perf_counter())
        return [round((t[i + 1] - t[i]) * 1e3, 3) for i in range(3)]
    for _ in range(5):
        step()
    plain = step()
    ctx.profile(True)
    timed = step()
    tl = ctx.profile_timeline()
    ctx.profile(False)
    t0 = min(r[2] for r in tl)
    print(json.dumps({"case": "timeline", "host_ms_per_call": plain, "host_ms_per_call_with_timers": timed}))
    for name, lane, a, e in sorted(tl, key=lambda r: r[2]):
        print(json.dumps({"name": name, "lane": lane, "start_ms": round(a - t0, 4), "end_ms": round(e - t0, 4)}))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the 8-, 216- and 512-atom cells")
    ap.add_argument("--case", default=None, choices=["projectors", "loewdin", "timeline"],
                    help="run one small case of a single path instead of the benchmark (for profiling)")
    ap.add_argument("--case-states", type=int, default=512)
    ap.add_argument("--case-atoms", type=int, default=128)
    args = ap.parse_args()
    if args.case == "projectors":
        run_case_projectors(args)
        return
    if args.case == "loewdin":
        run_case_loewdin(args)
        return
    if args.case == "timeline":
        run_case_timeline(args)
        return
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def geometry_summary(basis) -> dict:
    """Column / slot counts of the pruned FFT (mirrors the context's map build)."""
    import numpy as np
    m = basis.mill[: basis.ngw].astype(np.int64)
    full = np.concatenate([m, -m[1:]]) if basis.geq0 else np.concatenate([m, -m])
    cols = {}
    for gx, gy, gz in full.tolist():
        cols.setdefault((gx, gy), []).append(gz)
    gxs = sorted({k[0] for k in cols})
    ncol = 0
    nent = 0
    for gx in range(gxs[0], gxs[-1] + 1):
        gys = [k[1] for k in cols if k[0] == gx]
        if not gys:
            continue
        for gy in range(min(gys), max(gys) + 1):
            z = cols.get((gx, gy))
            ncol += 1
            if z:
                nent += max(z) - min(z) + 1
    return {"nr": basis.nr, "ncol": ncol, "nslot": gxs[-1] - gxs[0] + 1, "nent": nent, "ngw": basis.ngw}


if __name__ == "__main__":
    main()
