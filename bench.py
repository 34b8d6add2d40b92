#!/usr/bin/env python3
"""Benchmark of the implicit ADI step of the linearised single-Fourier-mode
solver (src/impdrv3d.f90) on one GB300.

Headline workload: a parallel compressible shear layer on a 512 x 256 grid
(x periodic, y stretched; u = (1 + tanh y)/2, T by Crocco-Busemann, Ma 0.8,
Re 500), spanwise wavenumber beta 0.2, frequency omega 0.05, local time
stepping at CFL 20, seeded 1e-6 disturbance in a Gaussian window.  A step is
one implicit step with one corrector (impl 1, niter 1): RHS, xi sweep, eta
sweep, update, on factors formed at the first step.  Inputs are synthetic
(lns3d_gb300.cases.shear_layer); the working set of a step (operators 131 MB,
two factored LHS of 262 MB each) is larger than L2.

One JSON line on stdout (rank 0):
  value        FP64 grid-point-steps per second of the drop-in step, all GPUs
  mixed        the same with FP32 LHS factors and sweeps (FP64 RHS, residual
               and update)
  converge     steps and time to a 1e-10 residual from the initial
               disturbance, FP64 and mixed, and the final state difference
  e2e          the FP64 step through the host-pointer C-ABI call
               (lns_step3d): disturbance copied from pinned host memory and
               back every step, inside the timed region
  roofline     the dominant kernel (a sweep) against the measured HBM copy
               bandwidth, and beside it against the measured FP64 rate
  cpu_baseline the oracle restatement of the step (OpenMP over all host
               cores) on a bounded sample of the same workload
  isolated_solve  the batched complex block-penta solve on its own (512
               lines x 256 rows, cpenta2bc factor + solve)

--impl reference times only the CPU path (the reference's Fortran cannot be
built without a Fortran compiler; its restatement stands in) and prints its
line.  Multi-GPU (torchrun): independent replicas, one per GPU; no
collective on the data path.
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

# ---- headline: the 3D step
NX, NY = 512, 256
PTS3 = NX * NY
CFL3 = 20.0
# algorithmic HBM bytes per grid point of each phase (FP64):
#   RHS     v, vold 160 B + operators 984 B (Ah Bh Dh Dhi 100 doubles, V 18,
#           the 4 used 3D terms, dtl) + r write 80 B            = 1224 B
#   xi sweep (periodic) factors 2000 B + border columns W 800 B + r read
#           and write 160 B                                       = 2960 B
#   eta sweep factors 2000 B + r read and write 160 B            = 2160 B
#   update  v read and write 160 B + r read 80 B                 =  240 B
PHASE_BYTES = {"rhs": 1224, "xsweep": 2960, "ysweep": 2160, "update": 240}
# complex multiply-adds per point of a sweep (8 flops each): D^-1 25, lower
# blocks 50, upper blocks 50; the periodic border correction +50
PHASE_FLOPS = {"xsweep": 8 * 175, "ysweep": 8 * 125}
# per kernel segment (lns_ctx3d_profile): algorithmic bytes and flops per
# grid point of one launch, FP64
#   rhs      grad1 + rhs + resid: v, vold, dv/dxi 240 B + operators 984 B + r 80 B
#            (about 510 FMA: operator products 200, derivatives 240, viscous
#            and 3D terms 50, rbe and residual 20)
#   x_scale  D^-1 400 B + r read and write 160 B            (25 complex FMA)
#   x_fwd    the xi lines in row pairs: the even rows' pass (F1 400 B, two
#            right-hand sides read and one written, on half the rows: 320 B,
#            12.5 complex FMA) + the paired recurrence (two blocks 800 B + s
#            read 80 B + yh write 80 B, 50 complex FMA)
#   x_bwd    as x_fwd with B1 and the backward blocks
#   x_fill   the periodic border: W 800 B + x read, write 160 B (50 complex
#            FMA), and per line S^-1, A21 (the border unknowns)
#   y_*      row by row: two blocks 800 B + 160 B (50 complex FMA); the
#            scaling as x_scale
#   update   v read, write 160 B + r 80 B
KERNEL_BYTES = {"rhs": 1304, "x_scale": 560, "x_fwd": 1280, "x_fill": 960, "x_bwd": 1280, "y_scale": 560,
                "y_fwd": 960, "y_bwd": 960, "update": 240}
KERNEL_FLOPS = {"rhs": 1020, "x_scale": 200, "x_fwd": 500, "x_fill": 400, "x_bwd": 500, "y_scale": 200,
                "y_fwd": 400, "y_bwd": 400}
KERNEL_NAMES = {"x_fwd": "even_kernel<0> + pair_chain_kernel<0, 0> (xi forward recurrence in row pairs)",
                "x_bwd": "even_kernel<1> + pair_chain_kernel<1, 0> (xi backward recurrence in row pairs)",
                "y_fwd": "chain_fwd_kernel<cd, 0> (eta forward recurrence)",
                "y_bwd": "chain_bwd_kernel<cd, 0> (eta backward recurrence)",
                "rhs": "grad1_kernel + rhs_kernel + resid_kernel"}
# DRAM bytes (read + write) per launch from ncu captures on this workload:
# the xi segments (even pass + paired recurrence) from
# profiles/pair_chain_kernel_cd_xsweep_512x256.md, the eta backward
# recurrence from profiles/chain_bwd_kernel_cd_sweeps_512x256.md
KERNEL_TRAFFIC = {"x_fwd": 43.721984e6 + 6912 + 129.308928e6 + 2.872320e6,
                  "x_bwd": 43.753728e6 + 1536 + 129.341696e6 + 2.977024e6,
                  "y_bwd": 130.674432e6 + 2.793728e6}
KERNELS_PER_STEP = 16  # bc (predictor), grad1, rhs, resid, xi sweep (7: scale, two even passes, two paired
#                       recurrences, border, correction), eta sweep (3), add, bc
# whole-step model of the linearised step with stored factors, per grid point
# and step: RHS 1224 B (v, vold 160 B, frozen operators 984 B, r 80 B), xi
# sweep 2160 B (factors 2000 B, r read and write 160 B), eta sweep 2240 B
# (factors 2000 B, r read 80 B, v read and write 160 B); about 1 kflop for
# the RHS and 1 kflop for each directional solve.  The periodic fill of the
# xi lines (1600 B and 800 flops more per point) is outside this model.
STEP_BYTES, STEP_FLOPS = 5624, 3000

# ---- secondary: the isolated batched solve
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


def fp64_probe():
    """Live FP64 FMA rate of this GPU (TFLOP/s) from the probe library that
    lns3d_gb300/_build.py builds beside the product library."""
    from lns3d_gb300 import _build

    L = ctypes.CDLL(os.path.join(_build.LIBDIR, _build.PROBE_NAME))
    L.lns_probe_fp64_tflops.restype = ctypes.c_double
    L.lns_probe_fp64_tflops.argtypes = []
    return L.lns_probe_fp64_tflops()


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


def max_over_ranks(torch, x, dev, world):
    """The largest x over the replicas (the timing rule of a multi-GPU run:
    each rank times its own replica, the job takes as long as the slowest);
    x itself on one rank."""
    if world <= 1:
        return x
    t = torch.tensor([float(x)], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


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
    total_ms = max_over_ranks(torch, total_ms, dev, world)
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
        return world * PTS / max_over_ranks(torch, max(t), dev, world)
    return PTS / statistics.mean(t)


def step3d_cpu(steps, warm=1):
    """The oracle restatement of the step built with OpenMP over grid rows and
    lines (oracle/liborc_omp.so), all host cores, on the headline workload;
    returns seconds per step over `steps` steps after `warm` steps (the first
    of which forms and factors the LHS)."""
    import numpy as np

    import oracle
    from lns3d_gb300.cases import shear_layer

    from oracle.adi3d import Oracle3D

    lib = oracle.orc_omp()
    case = shear_layer(nx=NX, ny=NY, seed=0)
    orc = Oracle3D(case, cflmax=CFL3, loctime=1, lib=lib)
    v = np.asfortranarray(case["v"].copy())
    for _ in range(warm):
        orc.step(v)
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.step(v)
    return (time.perf_counter() - t0) / steps


def cpu_baseline3d(steps):
    t = step3d_cpu(steps)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": PTS3 / t, "unit": "grid-pt-steps/s", "cores": cores, "kind": "port",
            "sample": "%d implicit steps (niter 1) of the 512x256 shear-layer case after the factoring step, "
                      "%.1f ms/step; restatement of impdrv3d + cpenta2p/cpenta1bc, -O3 -fopenmp" % (steps, t * 1e3)}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    t = step3d_cpu(steps, warm=max(1, min(args.warmup, 2)))
    wall = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    value = PTS3 / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "grid-pt-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic", "config": config3(world),
            "cpu_baseline": {"value": value, "unit": "grid-pt-steps/s", "cores": cores, "kind": "port",
                             "sample": "%d implicit steps of the 512x256 case on %d host threads (the reference's "
                                       "Fortran has no compiler here; its C restatement, -O3 -fopenmp)"
                                       % (steps, cores)},
            "e2e": {"value": value, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))
    return 0


METRIC = "ADI grid-pt-steps/s (linearised 3D implicit step, FP64 drop-in; mixed beside)"


def config3(world):
    return {"workload": "impdrv3d-shear-layer-512x256-beta0.2-omega0.05-niter1", "nx": NX, "ny": NY,
            "beta": 0.2, "omega": 0.05, "cfl": CFL3, "loctime": 1, "niter": 1,
            "parallelism": "replicas" if world > 1 else "single",
            "grid": "x uniform on [0, 5.5] (periodic); y = 10 sinh(3 (2 eta - 1)) / sinh(3), metrics exact "
                    "for the mapping",
            "timed": "K steps after warm-up from the seeded disturbance (the run to 1e-10 is the converge leg)",
            "l2": "working set larger than L2 (operators 131 MB + two factored LHS 262 MB each per step)"}


def time_steps(torch, drv, v, K, stream, totres=None):
    """K steps of one step each, CUDA events around every step; returns
    (total ms, sorted per-step ms)."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(K):
        ev[s][0].record(stream)
        drv.step(v, nsteps=1, niter=1, totres=None if totres is None else totres[s:])
        ev[s][1].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), sorted(a.elapsed_time(b) for a, b in ev)


def converge(torch, drv, v0, tol=1e-10, max_steps=2000, chunk=100):
    """Steps from v0 until the residual is <= tol (or max_steps); returns
    (steps, ms, residual history, final v)."""
    v = v0.clone()
    res = torch.zeros(max_steps, dtype=torch.float64, device=v.device)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    done = 0
    hit = None
    while done < max_steps and hit is None:
        n = min(chunk, max_steps - done)
        drv.step(v, nsteps=n, niter=1, totres=res[done:])
        done += n
        r = res[:done].cpu()
        below = (r <= tol).nonzero()
        if below.numel():
            hit = int(below[0]) + 1
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return (hit if hit is not None else -1), ms, done, res[:done].cpu().numpy(), v


def percentile(xs, q):
    return xs[min(len(xs) - 1, int(round(q * (len(xs) - 1))))]


def run_isolated(torch, dev, L, sp, stream, rank, world, W, K, with_cpu=False):
    """The isolated batched solve (cpenta2bc code 2, FP64) and its mixed
    form; each step solves its own pristine batch resident in HBM.  With
    with_cpu, the reference's own cpenta2bc (translated) on the host cores
    beside it."""
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
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for s in range(K):
        ev[s][0].record(stream)
        solve(*batches[W + s])
        ev[s][1].record(stream)
    torch.cuda.synchronize()
    per_step = sorted(a.elapsed_time(b) for a, b in ev)
    assert torch.isfinite(torch.view_as_real(batches[W][1])).all()
    fp64_x = batches[W][1].clone()
    del batches
    mixed = run_mixed(torch, dev, L, sp, stream, rank, world, W, K, fp64_x)
    ms = statistics.mean(per_step)
    return {"workload": "cpenta2bc-512lines-256rows-complex-factor+solve", "value": PTS / (ms / 1e3),
            "unit": "grid-pt/s", "ms_per_step": ms,
            "latency_ms": {"p50": percentile(per_step, 0.5), "p99": percentile(per_step, 0.99)},
            "bytes_per_pt": BYTES_PER_PT, "flops_per_pt": FLOPS_PER_PT,
            "hbm_gbs": BYTES_PER_PT * PTS / (ms / 1e3) / 1e9,
            "fp64_tflops": FLOPS_PER_PT * PTS / (ms / 1e3) / 1e12, "mixed": mixed,
            "cpu_baseline": time_reference_cpu() if with_cpu else None}


def run_impdrv2d(torch, dev, steps, with_cpu):
    """The nonlinear 2D step (src/impdrv.f90) on its benchmark case: an Oseen
    vortex in a uniform stream, 128 x 128, Ma 0.5, Re 1000, global time step
    at CFL 1 (lns3d_gb300.cases.vortex2d).  Each step forms and factors both
    LHS, as the reference does; FP64 throughout."""
    import lns3d_gb300 as g
    from lns3d_gb300.cases import vortex2d

    c = vortex2d(nx=128, ny=128, seed=0)
    drv = g.ImpDrv2D(c["params"], c["metrics"], c["bnt"], c["pot"], cflmax=1.0, loctime=0)
    v = torch.from_numpy(c["v"].ravel(order="F")).to(dev)
    drv.itrbc(v)
    drv.step(v, nsteps=3)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    total, per = time_steps(torch, drv, v, steps, stream)
    pts = 128 * 128
    out = {"workload": "impdrv-oseen-vortex-128x128-Ma0.5-Re1000-cfl1",
           "grid": "[-10, 10]^2, x uniform (periodic), y = 10 tanh(2 (2 eta - 1)) / tanh(2); metrics by the "
                   "reference pre-processor's differencing (lns3d_gb300.pre)",
           "value": pts * steps / (total / 1e3),
           "unit": "grid-pt-steps/s", "ms_per_step": total / steps, "dtype": "f64",
           "latency_ms": {"p50": percentile(per, 0.5), "p99": percentile(per, 0.99)},
           "launches_per_step": 12, "cpu_baseline": None}
    # the nonlinear 2D step's model per grid point and step: 1856 B (v, vold,
    # metrics, the operator hand-off between phases, r) and 5.5 kflop (RHS
    # and operators 2 kflop, two factor-and-solve passes of about 850 FMA
    # per row each), against the measured copy bandwidth and the live FP64
    # rate
    rate = out["value"]
    hbm_peak, peak_kind = peaks()
    fp64_peak = fp64_probe()
    out["roofline"] = {"bound": "fp64", "bytes_per_pt": 1856, "flops_per_pt": 5500,
                       "hbm_gbs": rate * 1856 / 1e9, "hbm_frac": rate * 1856 / 1e9 / hbm_peak,
                       "fp64_tflops": rate * 5500 / 1e12, "fp64_frac": rate * 5500 / 1e12 / fp64_peak,
                       "peak_source": peak_kind + " HBM copy; live FP64 DFMA stream"}
    if with_cpu:
        from oracle.impdrv2d import Oracle2D
        import oracle

        o = Oracle2D(c, cflmax=1.0, loctime=0, lib=oracle.orc_omp())
        vh = c["v"].copy(order="F")
        o.itrbc(vh)
        o.step(vh)
        n = 10
        t0 = time.perf_counter()
        for _ in range(n):
            o.step(vh)
        t = (time.perf_counter() - t0) / n
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        out["cpu_baseline"] = {"value": pts / t, "unit": "grid-pt-steps/s", "cores": cores, "kind": "port",
                               "sample": "%d steps of the 128x128 vortex case, %.1f ms/step; restatement of "
                                         "impdrv + penta2p/penta1bc, -O3 -fopenmp" % (n, t * 1e3)}
    return out


def batch_problems(P=64, seed=4):
    """The batched workload: 64 linearised shear-layer problems, beta on a
    uniform grid of [0, 0.4] and omega on [0.01, 0.1] (8 x 8), grid sizes
    drawn by seed from nx in {128, 192, 256, 384, 512}, ny in {64, 96, 128,
    192, 256}."""
    import numpy as np

    from lns3d_gb300.cases import shear_layer

    rng = np.random.default_rng(seed)
    side = int(round(P ** 0.5))
    betas = np.linspace(0.0, 0.4, side)
    omegas = np.linspace(0.01, 0.1, side)
    out = []
    for k in range(P):
        nx = int(rng.choice([128, 192, 256, 384, 512]))
        ny = int(rng.choice([64, 96, 128, 192, 256]))
        out.append(shear_layer(nx=nx, ny=ny, beta=float(betas[k // side]), omega=float(omegas[k % side]), seed=k))
    return out


def run_batch(torch, with_cpu, max_steps=2000, tol=1e-10):
    """All 64 problems to a 1e-10 residual in one batch, lines per CTA
    autotuned, twice: in FP64 (the drop-in arithmetic) and in the mixed mode
    (FP64 residual, FP32 scaled factors and sweeps).  The headline of the leg
    is the mixed run; the FP64 run of the same problems gives the mixed/FP64
    ratio on equal work and the mixed results' distance from the FP64 ones."""
    import numpy as np

    import lns3d_gb300 as g

    probs = batch_problems()
    pts = np.array([c["params"]["nx"] * c["params"]["ny"] for c in probs])

    def one(precision):
        t0 = time.perf_counter()
        batch = g.Batch3D(probs, cflmax=CFL3, loctime=1, precision=precision)
        w = batch.tune()
        setup = time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        steps, res = batch.run(max_steps=max_steps, tol=tol, check_every=25)
        wall = time.perf_counter() - t0
        states = [batch.state(k) for k in range(len(probs))]
        nbytes = int(batch.device_bytes)
        batch.close()
        conv = steps > 0
        done_pts = float((pts * np.where(conv, steps, max_steps)).sum())
        return dict(steps=steps, conv=conv, states=states, wall=wall, setup=setup, w=w, bytes=nbytes,
                    value=done_pts / wall)

    f64 = one(g.adi3d.FP64)
    mix = one(g.adi3d.MIXED)
    both = f64["conv"] & mix["conv"]
    # time to the tolerance on the problems that reach it in both modes: the
    # wall time of each run scaled by that set's share of its point-steps
    def share(r):
        done = pts * np.where(r["conv"], r["steps"], max_steps)
        return float((pts * r["steps"])[both].sum() / done.sum()) * r["wall"]

    err = max((float(np.abs(mix["states"][k] - f64["states"][k]).max() / np.abs(f64["states"][k]).max())
               for k in np.flatnonzero(both)), default=None)
    conv = mix["conv"]
    steps = mix["steps"]
    out = {"workload": "batch-64-shear-layers-beta0-0.4-omega0.01-0.1-uneven-grids-mixed-to-1e-10",
           "problems": len(probs), "grid_points": int(pts.sum()), "converged": int(conv.sum()),
           "steps_min": int(steps[conv].min()) if conv.any() else None,
           "steps_max": int(steps[conv].max()) if conv.any() else None,
           "wall_s": mix["wall"], "setup_s": mix["setup"], "value": mix["value"], "unit": "grid-pt-steps/s",
           "lines_per_cta": mix["w"], "device_bytes": mix["bytes"],
           "not_converged": [int(k) for k in np.flatnonzero(~conv)],
           "fp64": {"value": f64["value"], "wall_s": f64["wall"], "converged": int(f64["conv"].sum()),
                    "lines_per_cta": f64["w"], "device_bytes": f64["bytes"]},
           "mixed_vs_fp64": {"throughput_ratio": mix["value"] / f64["value"],
                             "converged_in_both": int(both.sum()),
                             "same_steps_in_both": int((f64["steps"][both] == mix["steps"][both]).sum()),
                             "time_to_tol_ratio": share(f64) / share(mix) if both.any() else None,
                             "max_state_rel_diff": err},
           "cpu_baseline": None}
    if with_cpu:
        import oracle
        from oracle.adi3d import Oracle3D

        lib = oracle.orc_omp()
        t = 0.0
        n = 0
        for c in probs[:8]:
            o = Oracle3D(c, cflmax=CFL3, loctime=1, lib=lib)
            v = np.asfortranarray(c["v"].copy())
            o.step(v)
            t0 = time.perf_counter()
            o.step(v)
            o.step(v)
            t += time.perf_counter() - t0
            n += 2 * c["params"]["nx"] * c["params"]["ny"]
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        out["cpu_baseline"] = {"value": n / t, "unit": "grid-pt-steps/s", "cores": cores, "kind": "port",
                               "sample": "2 steps of each of the first 8 problems, serially, OpenMP inside each"}
    return out


def serve_stream(n, rate=50.0, seed=5):
    """The served stream: n linearised solve requests with Poisson arrivals
    at `rate` per second, beta ~ U[0, 0.5], omega ~ U[0.01, 0.15], nx and ny
    log-uniform in [64, 1024] x [64, 512] (multiples of 16), tolerance 1e-10;
    the shear-layer mean flow of the other legs on each request's grid."""
    import numpy as np

    from lns3d_gb300.cases import shear_layer

    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for k in range(n):
        nx = int(np.clip(16 * round(np.exp(rng.uniform(np.log(64), np.log(1024))) / 16), 64, 1024))
        ny = int(np.clip(16 * round(np.exp(rng.uniform(np.log(64), np.log(512))) / 16), 64, 512))
        reqs.append((float(t[k]), nx, ny, float(rng.uniform(0.0, 0.5)), float(rng.uniform(0.01, 0.15)), k))
    return reqs


def run_serve(torch, n_requests=100, rate=50.0, tol=1e-10, max_steps=2000, serial_every=10):
    """The serving leg: a prefix of the stream through lns_server3d (mixed
    precision, continuous batching, 64 slots, 64 GiB budget) in real time,
    and every serial_every-th request of the same prefix solved one at a time
    by the FP64 drop-in step, for the serial comparison (solves per second of
    the sample, the same tolerance and step limit)."""
    import numpy as np

    import lns3d_gb300 as g
    from lns3d_gb300.cases import shear_layer

    reqs = serve_stream(n_requests, rate)
    cases = [shear_layer(nx=nx, ny=ny, beta=beta, omega=omega, seed=k) for _, nx, ny, beta, omega, k in reqs]
    srv = g.Server3D(64 << 30, max_slots=64, precision=g.adi3d.MIXED)
    pending = [(r[0], c) for r, c in zip(reqs, cases)]
    ids = []
    t0 = time.perf_counter()
    while pending or any(srv.poll(i)["state"] in ("queued", "running") for i in ids):
        now = time.perf_counter() - t0
        while pending and pending[0][0] <= now:
            ids.append(srv.submit(pending.pop(0)[1], tol=tol, max_steps=max_steps, cflmax=CFL3))
        running, queued = srv.tick(25)
        if not running and not queued and pending:
            time.sleep(max(0.0, pending[0][0] - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    polls = [srv.poll(i) for i in ids]
    lat = np.array(sorted(p["latency_s"] for p in polls))
    done = sum(p["state"] == "done" for p in polls)
    pts = np.array([c["params"]["nx"] * c["params"]["ny"] for c in cases], dtype=np.float64)
    served_pt_steps = float(sum(p["steps"] * n for p, n in zip(polls, pts)))
    srv.close()
    # serial FP64 drop-in solves of every serial_every-th request
    ser, ser_pt_steps = [], 0.0
    for k in range(0, n_requests, serial_every):
        c = cases[k]
        d = g.ImpDrv3D(c["params"], c["metrics"], c["vm"], cflmax=CFL3, loctime=1, precision=g.adi3d.FP64)
        v = torch.from_numpy(c["v"].ravel(order="F")).cuda()
        res = torch.zeros(max_steps, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ts = time.perf_counter()
        steps = 0
        while steps < max_steps:
            d.step(v, nsteps=25, totres=res[steps:])
            steps += 25
            if float(res[steps - 1].item()) <= tol:
                break
        ser.append(time.perf_counter() - ts)
        ser_pt_steps += steps * pts[k]
        d.close()
    return {"workload": "serve-%d-of-1000-requests-poisson-%g-per-s-mixed-to-1e-10" % (n_requests, rate),
            "requests": n_requests, "converged": int(done), "wall_s": wall, "solves_per_s": n_requests / wall,
            "pt_steps_per_s": served_pt_steps / wall,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "serial_fp64": {"sample": "every %dth request (%d solves)" % (serial_every, len(ser)),
                            "mean_solve_s": float(np.mean(ser)), "solves_per_s": len(ser) / float(np.sum(ser)),
                            "pt_steps_per_s": ser_pt_steps / float(np.sum(ser))}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-pointer end-to-end leg")
    ap.add_argument("--no-converge", action="store_true", help="skip the runs to a 1e-10 residual")
    ap.add_argument("--no-isolated", action="store_true", help="skip the isolated batched-solve leg")
    ap.add_argument("--no-2d", action="store_true", help="skip the nonlinear 2D step leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 64-problem leg")
    ap.add_argument("--serve-requests", type=int, default=100,
                    help="requests of the served stream to run (the stream has 1000); 0 skips the leg")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import lns3d_gb300 as g
    from lns3d_gb300.cases import shear_layer

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

    case = shear_layer(nx=NX, ny=NY, seed=rank)
    v0 = torch.from_numpy(case["v"].ravel(order="F")).to(dev)

    def make(precision):
        t0 = time.perf_counter()
        d = g.ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=CFL3, loctime=1, precision=precision)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        v = v0.clone()
        d.step(v, nsteps=1)   # forms and factors both LHS
        torch.cuda.synchronize()
        return d, v, {"operators_ms": (t1 - t0) * 1e3, "first_step_ms": (time.perf_counter() - t1) * 1e3}

    # ---- FP64 drop-in step
    d64, v64, setup64 = make(g.adi3d.FP64)
    for _ in range(W):
        d64.step(v64, nsteps=1)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = Clocks(local)
    total_ms, per_step = time_steps(torch, d64, v64, K, stream)
    clocks = clk.stop()
    total_ms = max_over_ranks(torch, total_ms, dev, world)
    if world > 1:
        torch.distributed.barrier()
    value = world * PTS3 * K / (total_ms / 1e3)

    # per-phase kernel times (events on the launching stream, separate pass)
    d64.profile(True)
    time_steps(torch, d64, v64, K, stream)
    phases64, ncorr, seg64 = d64.profile_read()
    d64.profile(False)
    ph64 = {k: v / ncorr for k, v in phases64.items()}
    kern64 = {k: v / ncorr for k, v in seg64.items()}

    # ---- mixed step
    d32, v32, setup32 = make(g.adi3d.MIXED)
    for _ in range(W):
        d32.step(v32, nsteps=1)
    torch.cuda.synchronize()
    total32, per32 = time_steps(torch, d32, v32, K, stream)
    d32.profile(True)
    time_steps(torch, d32, v32, K, stream)
    phases32, n32, seg32 = d32.profile_read()
    d32.profile(False)
    ph32 = {k: v / n32 for k, v in phases32.items()}
    kern32 = {k: v / n32 for k, v in seg32.items()}
    total32 = max_over_ranks(torch, total32, dev, world)
    mixed = {"value": world * PTS3 * K / (total32 / 1e3), "ms_per_step": total32 / K,
             "latency_ms": {"p50": percentile(per32, 0.5), "p99": percentile(per32, 0.99)},
             "phase_ms": ph32, "kernel_ms": kern32, "setup": setup32, "device_bytes": int(d32.device_bytes)}

    # ---- to a 1e-10 residual from the initial disturbance
    conv = None
    if not args.no_converge:
        a = converge(torch, g.ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=CFL3, loctime=1,
                                       precision=g.adi3d.FP64), v0)
        b = converge(torch, g.ImpDrv3D(case["params"], case["metrics"], case["vm"], cflmax=CFL3, loctime=1,
                                       precision=g.adi3d.MIXED), v0)
        n = min(len(a[3]), len(b[3]))
        diff = float((a[4] - b[4]).abs().max() / a[4].abs().max())
        conv = {"tol": 1e-10, "max_steps": 2000,
                "fp64": {"steps": a[0], "ms": a[1], "steps_run": a[2], "final_res": float(a[3][-1]),
                         "pt_steps_per_s": PTS3 * a[2] / (a[1] / 1e3)},
                "mixed": {"steps": b[0], "ms": b[1], "steps_run": b[2], "final_res": float(b[3][-1]),
                          "pt_steps_per_s": PTS3 * b[2] / (b[1] / 1e3)},
                "mixed_vs_fp64_state_rel_diff": diff,
                "mixed_vs_fp64_res_rel_diff_max": float(np.max(np.abs(a[3][:n] - b[3][:n]) / a[3][:n])),
                "time_to_tol_speedup": (a[1] / b[1]) if a[0] > 0 and b[0] > 0 else None}

    # ---- end to end through the host-pointer C ABI
    e2e = None
    if not args.no_e2e:
        host_v = torch.from_numpy(case["v"].ravel(order="F")).pin_memory()
        hv = host_v.numpy()
        d64.step(hv, nsteps=1)
        ke = max(3, min(K, 10))
        t = []
        for _ in range(ke):
            t0 = time.perf_counter()
            d64.step(hv, nsteps=1)
            t.append(time.perf_counter() - t0)
        tm = statistics.mean(t)
        tm = max_over_ranks(torch, tm, dev, world)
        e2e = {"value": world * PTS3 / tm, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 5 * PTS3 * 16,
               "d2h_bytes_per_step": 5 * PTS3 * 16 + 8, "ms_per_step": tm * 1e3}

    # ---- the isolated batched solve
    iso = None
    if not args.no_isolated:
        del d32
        iso = run_isolated(torch, dev, L, sp, stream, rank, world, 3, max(3, min(K, 10)),
                           rank == 0 and not args.no_cpu_baseline)

    legb = None
    if not args.no_batch:
        legb = run_batch(torch, rank == 0 and not args.no_cpu_baseline)

    legs = None
    if args.serve_requests > 0:
        legs = run_serve(torch, n_requests=args.serve_requests)

    leg2d = None
    if not args.no_2d:
        leg2d = run_impdrv2d(torch, dev, max(10, K), rank == 0 and not args.no_cpu_baseline)

    hbm_peak, peak_kind = peaks()
    fp64_peak = fp64_probe()
    # the dominant kernel: the xi forward recurrence (chain_fwd_kernel<cd, 1>)
    dom = max(kern64, key=lambda k: kern64[k])
    achieved = KERNEL_BYTES[dom] * PTS3 / (kern64[dom] / 1e3) / 1e9
    fp64_achieved = KERNEL_FLOPS.get(dom, 0) * PTS3 / (kern64[dom] / 1e3) / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline3d(8)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "grid-pt-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic", "config": config3(world),
            "latency_ms": {"p50": percentile(per_step, 0.5), "p99": percentile(per_step, 0.99)},
            "phase_ms": ph64, "kernel_ms": kern64, "setup": setup64, "device_bytes": int(d64.device_bytes),
            "mixed": mixed, "converge": conv, "e2e": e2e,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": KERNEL_TRAFFIC.get(dom), "peak_source": peak_kind,
                         "kernel": KERNEL_NAMES.get(dom, dom), "kernel_ms": kern64[dom],
                         "bytes_per_pt": KERNEL_BYTES[dom]},
            "roofline_fp64": {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                              "frac": fp64_achieved / fp64_peak, "flops_per_pt": KERNEL_FLOPS.get(dom, 0),
                              "peak_source": "measured live: DFMA stream on every SM (lns_probe_fp64_tflops)"},
            "roofline_step": {"bytes_per_pt": STEP_BYTES, "flops_per_pt": STEP_FLOPS,
                              "hbm_gbs": value * STEP_BYTES / 1e9, "hbm_frac": value * STEP_BYTES / 1e9 / hbm_peak,
                              "fp64_tflops": value * STEP_FLOPS / 1e12,
                              "fp64_frac": value * STEP_FLOPS / 1e12 / fp64_peak,
                              "model": "whole step with stored factors (RHS 1224 B, xi sweep 2160 B, eta sweep "
                                       "2240 B per pt-step; 3 kflop), at the device-resident step rate"},
            "cpu_baseline": cpu,
            "isolated_solve": iso,
            "impdrv2d": leg2d,
            "batch": legb,
            "serve": legs,
            "gpu_launches": KERNELS_PER_STEP * K,
            "clocks": clocks,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
