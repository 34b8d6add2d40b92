#!/usr/bin/env python3
"""Benchmark of the batched block-pentadiagonal line solve.

Workload (the isolated batched solve): 512 independent complex lines of 256
block rows with 5x5 blocks, boundary-closure rows (cpenta2bc semantics),
factor + solve (code 2) per step.  Block entries have real and imaginary
parts uniform in [-1, 1] with +10*I on the diagonal blocks; right-hand sides
are standard normal.  Inputs are synthetic and seeded; every timed step
solves its own pristine batch resident in HBM (262 MB of matrix per batch,
larger than L2, so no flush is needed).

One JSON line on stdout (rank 0):
  value        grid points solved per second (rows x lines / step time), all GPUs
  e2e          the same through the host-pointer C-ABI call with pinned host
               buffers, host<->device copies inside the timed region
  roofline     HBM roofline of the solver kernel (algorithmic bytes / kernel
               time vs the measured copy bandwidth) and, beside it, the FP64
               roofline that binds it
  cpu_baseline the reference's own solver sources (translated to C, OpenMP
               over all host cores) on the same workload

--impl reference runs only the reference CPU path and prints its line.
Multi-GPU (torchrun): independent replicas, one per GPU; no collective on the
data path.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_ROWS, N_LINES = 256, 512
PTS = N_ROWS * N_LINES
MAT_EL = 125 * PTS           # complex elements
RHS_EL = 5 * PTS
CPLX = 16
# algorithmic HBM bytes per grid point, factor + solve: read and write the
# 2000 B matrix row, read and write the 80 B right-hand side
BYTES_PER_PT = 2 * 2000 + 2 * 80
# algorithmic FP64 flops per grid point (complex multiply-add = 8 flops):
# in-block LU 140, multipliers 150, Schur update 550, back substitution 60
FLOPS_PER_PT = 8 * (140 + 150 + 550 + 60)


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler run during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.idx = gpu_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_batch(torch, dev, seed):
    """One pristine batch on the device: mat(5,5,5,256,512), rhs(5,256,512)
    in the reference (Fortran) layout, as complex128 flat tensors."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    mat = torch.empty(MAT_EL * 2, dtype=torch.float64, device=dev).uniform_(-1.0, 1.0, generator=g)
    mat = torch.view_as_complex(mat.view(-1, 2))
    # diagonal blocks: slot k=3 (index 2), entries m == q: Fortran offset k + 5m + 25q
    idx = torch.arange(5, device=dev)
    diag = 2 + 5 * idx + 25 * idx
    m4 = mat.view(PTS, 125)
    m4[:, diag] += 10.0
    rhs = torch.randn(RHS_EL * 2, dtype=torch.float64, device=dev, generator=g)
    rhs = torch.view_as_complex(rhs.view(-1, 2))
    return mat, rhs


def time_reference_cpu(sample_reps=3):
    """The reference's own solver sources (translated by oracle/f77sub2c.py,
    -O3 -fopenmp) on the same workload, all host cores; falls back to the
    oracle restatement (single thread) where the translation was not built."""
    import numpy as np

    import oracle

    ncores = os.cpu_count() or 1
    R = oracle.ref(fast=True)
    rng = np.random.default_rng(7)
    mat0 = rng.uniform(-1, 1, (5, 5, 5, N_ROWS, N_LINES)) + 1j * rng.uniform(-1, 1, (5, 5, 5, N_ROWS, N_LINES))
    mat0[2] += 10 * np.eye(5)[:, :, None, None]
    mat0 = np.asfortranarray(mat0)
    rhs0 = np.asfortranarray(rng.standard_normal((5, N_ROWS, N_LINES)) + 1j * rng.standard_normal((5, N_ROWS, N_LINES)))
    times = []
    for _ in range(sample_reps):
        mat, rhs = mat0.copy(order="F"), rhs0.copy(order="F")
        t0 = time.perf_counter()
        if R is not None:
            R.ref_cpenta2bc(N_ROWS, N_LINES, 5, oracle.ptr(mat), oracle.ptr(rhs), 2)
        else:
            oracle.orc().orc_cpenta_bc(2, N_ROWS, N_LINES, oracle.ptr(mat), oracle.ptr(rhs), 2, 0)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    kind = "reference" if R is not None else "port"
    cores = int(os.environ.get("OMP_NUM_THREADS", ncores)) if R is not None else 1
    return {"value": PTS / t, "unit": "grid-pt/s", "cores": cores, "kind": kind,
            "sample": "%d full solves of the 512x256 complex workload (cpenta2bc code 2), median %.1f ms"
                      % (sample_reps, t * 1e3)}


def run_mixed(torch, dev, L, sp, stream, rank, world, W, K, fp64_x, refine=2):
    """Times the mixed-precision solve (lns_cpenta2bc_mixed_dev, code 2) and
    checks the first timed step's solution against the FP64 direct one."""
    batches = [make_batch(torch, dev, 1000 * rank + s) for s in range(W + K)]
    nbytes = L.lns_mixed_workspace_bytes(N_ROWS, N_LINES, 1, 0)
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    wp = ctypes.c_void_p(work.data_ptr())

    def solve(mat, rhs):
        rc = L.lns_cpenta2bc_mixed_dev(N_ROWS, N_LINES, 5, ctypes.c_void_p(mat.data_ptr()),
                                       ctypes.c_void_p(rhs.data_ptr()), 2, refine, wp, sp)
        if rc:
            raise RuntimeError(L.lns_last_error().decode())

    for s in range(W):
        solve(*batches[s])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for s in range(K):
        ev[s][0].record(stream)
        solve(*batches[W + s])
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    per_step = sorted(a.elapsed_time(b) for a, b in ev)
    total_ms = sum(per_step)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    x = batches[W][1]
    err = float((x - fp64_x).abs().max() / fp64_x.abs().max())
    return {"value": world * PTS * K / (total_ms / 1e3), "ms_per_step": total_ms / K,
            "latency_ms": {"p50": per_step[len(per_step) // 2], "p99": per_step[-1]},
            "refine_steps": refine, "rel_diff_vs_fp64_direct": err,
            "workspace_bytes": int(nbytes), "launches_per_step": 3 + 4 * refine + 3}


def run_e2e(torch, dev, L, rank, world, K):
    """Steps through the host-pointer entry point lns_cpenta2bc: each step
    copies the step's matrix and right-hand side from pinned host memory to
    the device, solves, and copies the factored matrix, the solution and the
    status word back."""
    host_mat = torch.empty(MAT_EL, dtype=torch.complex128).pin_memory()
    host_rhs = torch.empty(RHS_EL, dtype=torch.complex128).pin_memory()
    src = [make_batch(torch, dev, 50000 + 1000 * rank + s) for s in range(2)]
    host_src = [(m.cpu().pin_memory(), r.cpu().pin_memory()) for m, r in src]
    del src
    ke = max(2, min(K, 5))

    def e2e_step(s):
        m, r = host_src[s % 2]
        host_mat.copy_(m)
        host_rhs.copy_(r)
        t = time.perf_counter()
        rc = L.lns_cpenta2bc(N_ROWS, N_LINES, 5, ctypes.c_void_p(host_mat.data_ptr()),
                             ctypes.c_void_p(host_rhs.data_ptr()), 2)
        if rc:
            raise RuntimeError(L.lns_last_error().decode())
        return time.perf_counter() - t

    e2e_step(0)
    t = [e2e_step(s) for s in range(ke)]
    if world > 1:
        tt = torch.tensor([max(t)], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        return world * PTS / float(tt.item())
    return PTS / statistics.mean(t)


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    reps = max(1, args.steps)
    for _ in range(args.warmup):
        time_reference_cpu(1)
    t0 = time.perf_counter()
    cb = time_reference_cpu(reps)
    wall = time.perf_counter() - t0
    line = {"impl": "reference", "metric": "ADI grid-pt-steps/s (isolated batched complex block-penta solve)",
            "value": cb["value"], "unit": "grid-pt/s", "n_gpus": args.gpus, "steps": reps,
            "warmup": args.warmup, "ms_per_step": 1e3 * PTS / cb["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "cpenta2bc-512lines-256rows-complex-factor+solve", "lines": N_LINES,
                       "rows": N_ROWS, "nblk": 5, "code": 2},
            "cpu_baseline": {"value": cb["value"], "unit": "grid-pt/s", "cores": cb["cores"], "kind": cb["kind"],
                             "sample": cb["sample"]},
            "e2e": {"value": cb["value"], "unit": "grid-pt/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-pointer end-to-end leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import lns3d_gb300 as g

    rank, world, local = env_rank()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    L = g.lib()
    W, K = max(3, args.warmup), max(1, args.steps)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    # pristine batches: one per warm-up and timed step
    batches = [make_batch(torch, dev, 1000 * rank + s) for s in range(W + K)]
    torch.cuda.synchronize()

    def solve(mat, rhs):
        rc = L.lns_cpenta2bc_dev(N_ROWS, N_LINES, 5, ctypes.c_void_p(mat.data_ptr()),
                                 ctypes.c_void_p(rhs.data_ptr()), 2, sp)
        if rc:
            raise RuntimeError(L.lns_last_error().decode())

    for s in range(W):
        solve(*batches[s])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_all0 = torch.cuda.Event(enable_timing=True)
    e_all1 = torch.cuda.Event(enable_timing=True)
    e_all0.record(stream)
    for s in range(K):
        ev[s][0].record(stream)
        solve(*batches[W + s])
        ev[s][1].record(stream)
    e_all1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    total_ms = e_all0.elapsed_time(e_all1)
    per_step = sorted(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        torch.distributed.barrier()
    ms_per_step = total_ms / K
    value = world * PTS * K / (total_ms / 1e3)
    kern_ms = statistics.mean(per_step)

    assert torch.isfinite(torch.view_as_real(batches[W][1])).all()
    fp64_x = batches[W][1].clone()
    del batches

    # mixed precision: FP32 LU + two FP64 refinement steps, same workload;
    # the matrix is read only, so the batches are regenerated pristine
    mixed = None
    if not args.no_mixed:
        mixed = run_mixed(torch, dev, L, sp, stream, rank, world, W, K, fp64_x)

    # end to end: host-pointer C-ABI call from pinned host memory
    e2e_value = None if args.no_e2e else run_e2e(torch, dev, L, rank, world, K)

    hbm_peak, peak_kind = peaks()
    fp64_peak = L.lns_probe_fp64_tflops()  # measured live on this GPU
    achieved = BYTES_PER_PT * PTS / (kern_ms / 1e3) / 1e9
    fp64_achieved = FLOPS_PER_PT * PTS / (kern_ms / 1e3) / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = time_reference_cpu(3)
    if rank == 0:
        line = {
            "metric": "ADI grid-pt-steps/s (isolated batched complex block-penta solve)",
            "value": value, "unit": "grid-pt/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "cpenta2bc-512lines-256rows-complex-factor+solve", "lines": N_LINES,
                       "rows": N_ROWS, "nblk": 5, "code": 2, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (262 MB matrix per step, fresh batch each step)"},
            "latency_ms": {"p50": per_step[len(per_step) // 2],
                           "p99": per_step[min(len(per_step) - 1, int(round(0.99 * (len(per_step) - 1))))]},
            "e2e": None if e2e_value is None else {
                "value": e2e_value, "unit": "grid-pt/s",
                "h2d_bytes_per_step": (MAT_EL + RHS_EL) * CPLX,
                "d2h_bytes_per_step": (MAT_EL + RHS_EL) * CPLX + 4},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": None,
                         "peak_source": peak_kind, "kernel": "penta_bc_kernel<cd>",
                         "bytes_per_pt": BYTES_PER_PT},
            "roofline_fp64": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak,
                              "unit": "TFLOP/s", "frac": fp64_achieved / fp64_peak,
                              "flops_per_pt": FLOPS_PER_PT,
                              "peak_source": "measured live: DFMA stream on every SM (lns_probe_fp64_tflops)"},
            "cpu_baseline": cpu,
            "mixed": mixed,
            "gpu_launches": K,
            "clocks": clocks,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
