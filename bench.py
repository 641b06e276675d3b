"""Benchmark: batched 1-D TE+TM RCWA solves per second on GB300.

Workload (the headline batched configuration): one seeded grating-on-mirror structure -- a binary
grating (fill and depth uniform in 0.3..0.5, n = 1.46 / 1.0, period 0.574) on a 20-layer quarter-wave
mirror (n = 2.1 / 1.46 at 1.053, H first), substrate 1.46 -- swept over 4096 seeded points
(lambda uniform in 0.9..1.2, theta uniform in 50..70 degrees), each solved for TE and TM at M = 60
(N = 121). One step = the two sweeps = 8192 solves, all in FP64 (complex128).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      solves/s with inputs resident in device memory (the *_dev C entry point, both
           polarizations per call), timed with CUDA events on the engine's stream, L2 flushed between steps.
e2e        the same metric through the host-buffer C entry point (host -> device copy of the points
           and device -> host copy of all results inside the timed region).
roofline   the eigensolve stage (the dominant stage; for the grating's real permittivities its three
           Hermitian kernels): algorithmic FP64 flops per launch / its event-timed duration, against the
           FP64 peak measured here with cuBLAS DGEMM.
cpu_baseline  the CPU oracle (a C++ restatement of the reference's solve) on the host cores.
--impl reference  times that CPU implementation alone on the same workload definition.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20241203
N_POINTS = 4096
M = 60
PERIOD = 0.574
METRIC = "solves/s, batched 1-D TE+TM sweep (M=60, N=121), per-order efficiency error <= 1e-10 vs the FP64 CPU oracle"
WORKLOAD = ("batched 1-D TE+TM sweep, M=60 (N=121), binary grating on a 20-layer quarter-wave mirror, "
            "4096 seeded (lambda, theta) points x 2 polarizations per step")


# the absorbing variant of the grating (the general Hessenberg + shifted QR eigensolver instead of the
# Hermitian one): index 1.46 + 0.01i
LOSSY_RIDGE = complex(1.46, 0.01)


def workload(seed=SEED, n_points=N_POINTS, ridge=1.46):
    from stablercwa_gb300 import Layer, Stack
    rng = np.random.default_rng(seed)
    fill, depth = rng.uniform(0.3, 0.5), rng.uniform(0.3, 0.5)
    layers = [Layer.grating(depth, [0.0, fill * PERIOD, PERIOD], [ridge, 1.0])]
    for _ in range(10):
        layers.append(Layer.uniform(1.053 / (4 * 2.1), 2.1))
        layers.append(Layer.uniform(1.053 / (4 * 1.46), 1.46))
    stack = Stack(nI=1.0, nII=1.46, period=PERIOD, layers=layers)
    pts = np.stack([rng.uniform(0.9, 1.2, n_points), rng.uniform(50.0, 70.0, n_points)], axis=1)
    return stack, pts, {"fill": float(fill), "depth": float(depth)}


# DRAM bytes per matrix of the Hermitian eigensolve stage at n = 121 (blocked tridiagonalisation 22.0 MB,
# its tensor-core trailing updates and the back-transformation with their digit splits 8.5 MB, QL 0.3 MB,
# rotations on the real identity 1.2 MB, the rest 1.0 MB), from one ncu capture of every launch of one
# 4096-matrix eigensolve of this order
HERM_STAGE_DRAM_BYTES_PER_MATRIX_N121 = 33.0e6


HERM_STAGE_KERNELS = ("eigensolve stage: herm_panel_batch_kernel (blocked tridiagonalisation, FP64) + tensor-core "
                      "trailing updates + herm_ql_kernel + herm_apply_real_kernel (QL, FP64; its rotations on a real "
                      "identity in 64-bit fixed point on the integer pipes) + tensor-core back-transformation")


def herm_flops_text(n, rotations_per_matrix):
    vec = (f"QL rotations 6 n each ({rotations_per_matrix:.0f} per matrix measured)" if rotations_per_matrix > 0
           else "divide and conquer 8/3 n^3")
    return (f"Hermitian eigensolve at order {n}: tridiagonalisation 16/3 n^3, tridiagonal eigenvectors by {vec}, "
            f"back-transformation Q Y 4 n^3 (real flops per matrix)")


def herm_eig_flops(n, rotations_per_matrix):
    """Algorithmic real flops of one Hermitian eigensolve with eigenvectors: the Householder tridiagonalisation
    (16/3 n^3, LAPACK's zhetrd count), the tridiagonal eigenvectors (divide and conquer: about 8/3 n^3 for the
    merge products without deflation; or, when the QL iteration runs, 6 n per measured rotation, which the
    engine applies in fixed point on the integer pipes and counts at its FP64 equivalent), and the
    back-transformation of the real eigenvectors by Q (4 n^3)."""
    vec = 6 * n * rotations_per_matrix if rotations_per_matrix > 0 else (8 / 3) * n ** 3
    return (16 / 3) * n ** 3 + vec + 4 * n ** 3


def engine_flops_per_solve(n, pol, rotations_per_matrix, reduced=True):
    """FP64 flops of one solve of this stack (a grating over films) as the engine performs it: LU factor
    8/3 n^3, triangular solves 8 n^2 per right-hand side, GEMM 8 n^3.
    eigensolve   Hermitian (rotations_per_matrix > 0): herm_eig_flops;
                 general: 105 n^3.
    seams        reduced: grating over the first film, one LU with n right-hand sides (g is kept as its
                 factors and applied to vectors); top interface, one GEMM and one single-column LU. The reference's sequence: 5 LUs with n
                 right-hand sides, 1 single-column LU, 6 GEMMs.
    TM           general: the layer matrix [[1/eps]]^-1 B and V = [[1/eps]] W q, 2 GEMMs; Hermitian:
                 L^-1 B L^-H from the layer's constant parts (O(n^2)), then L^-H Y and L Y, 2 products with a
                 triangular factor (4 n^3 each)."""
    lu, tri, mm = (8 / 3) * n ** 3, 8 * n ** 3, 8 * n ** 3
    herm = not os.environ.get("RCWA_GB300_HERMITIAN", "").startswith("0")
    eig = herm_eig_flops(n, rotations_per_matrix) if herm else 105 * n ** 3
    if reduced:
        seams = (lu + tri) + (mm + lu + 8 * n ** 2)
    else:
        seams = 6 * lu + 5 * tri + 8 * n ** 2 + 6 * mm
    tm = 0 if pol == 0 else (2 * mm / 2 if herm else 2 * mm)
    return eig + seams + tm


def flops_per_solve(n, pol):
    """Flops of one solve of this stack counted op by op as the reference issues them: eigensolve
    105 n^3, LU factor 8/3 n^3, triangular solves 8 n^2 per right-hand side, GEMM 8 n^3. TE: 1 eig,
    6 LU (5 with n RHS, 1 with one), 6 GEMM; TM adds 2 LU with n RHS and 1 GEMM for the layer matrix
    and V."""
    eig = 105 * n ** 3
    if pol == 0:
        return eig + 6 * (8 / 3) * n ** 3 + 5 * 8 * n ** 3 + 8 * n ** 2 + 6 * 8 * n ** 3
    return eig + 8 * (8 / 3) * n ** 3 + 7 * 8 * n ** 3 + 8 * n ** 2 + 7 * 8 * n ** 3


# ------------------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------- CPU side

def cpu_sample_points(pts, count):
    idx = np.linspace(0, len(pts) - 1, count).astype(int)
    return pts[idx]


def cpu_rate(stack, pts, threads):
    """Oracle solves/s on `threads` host threads over TE + TM of the given points."""
    from oracle import oracle
    t0 = time.perf_counter()
    out = [oracle.solve1d_batch(stack, pts, M, pol, threads=threads) for pol in (0, 1)]
    dt = time.perf_counter() - t0
    return 2 * len(pts) / dt, out, dt


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores (the oracle port; the
    reference sources are not on the benchmark host), same workload definition and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    stack, pts, geo = workload()
    threads = os.cpu_count() or 1
    sample = cpu_sample_points(pts, args.ref_points)
    for _ in range(args.warmup):
        cpu_rate(stack, sample[: max(1, len(sample) // 8)], threads)
    times = []
    for _ in range(args.steps):
        _, _, dt = cpu_rate(stack, sample, threads)
        times.append(dt)
    solves = 2 * len(sample)
    value = solves * args.steps / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 (complex128)",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "points": N_POINTS, "M": M, "seed": SEED, **geo},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{len(sample)} of the {N_POINTS} points x TE+TM = {solves} solves per step"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------- GPU side

def fp64_peak_tflops(torch):
    """FP64 peak of this GPU, measured: cuBLAS DGEMM 4096^3 through torch, best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def replica_rate(world, units_per_rank, seconds, device="cpu"):
    """Whole-job rate of `world` replicas (one per rank, weak scaling): every rank's units over the slowest
    rank's time, the maximum taken over the ranks with one all-reduce (the replicas exchange no data)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return world * units_per_rank / seconds


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from stablercwa_gb300.engine import Engine, eig_rotations, launch_count

    if args.eig_group:
        os.environ["RCWA_GB300_EIG_GROUP"] = str(args.eig_group)
    stack, pts, geo = workload(n_points=args.points)
    n = 2 * M + 1
    P = len(pts)
    eng = Engine(device=local)
    est = torch.cuda.ExternalStream(eng.stream())
    d_pts = torch.tensor(pts, dtype=torch.float64, device="cuda")
    # both polarizations in one call (RCWA_TE_TM): TE rows 0..P-1, TM rows P..2P-1; the engine runs the
    # two sweeps concurrently on two streams
    out = {"R": torch.empty((2 * P, n, 2), dtype=torch.float64, device="cuda"),
           "T": torch.empty((2 * P, n, 2), dtype=torch.float64, device="cuda"),
           "DEr": torch.empty((2 * P, n), dtype=torch.float64, device="cuda"),
           "DEt": torch.empty((2 * P, n), dtype=torch.float64, device="cuda"),
           "status": torch.empty(2 * P, dtype=torch.int32, device="cuda")}
    ptrs = {k: v.data_ptr() for k, v in out.items()}
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def step():
        eng.solve1d_device(stack, d_pts.data_ptr(), P, M, 2, ptrs)

    peak = fp64_peak_tflops(torch)
    for _ in range(args.warmup):
        step()
    eng.synchronize()
    torch.cuda.synchronize()

    # ---- timed region: device-resident inputs
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = launch_count()
    eig_rotations()
    total_ms = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(est)
        step()
        e1.record(est)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    launches = launch_count() - launches0
    rotations = eig_rotations()
    clocks = sampler.stop()
    torch.cuda.synchronize()
    # per-kernel-kind breakdown from separate instrumented steps (the events around every launch cost a
    # little, so the timed steps above run without them)
    kstep = max(1, min(args.steps, 2))
    eng.set_kernel_timing(True)
    for _ in range(kstep):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        step()
        eng.synchronize()
    eig_busy_ms = eng.kernel_busy("eig")
    eig_ms, eig_launches = eng.kernel_time("eig")
    lu_ms, lu_launches = eng.kernel_time("lu")
    gemm_ms, gemm_launches = eng.kernel_time("gemm")
    eng.set_kernel_timing(False)
    eig_rotations()
    solves_per_step = 2 * P
    value = replica_rate(world, solves_per_step * args.steps, total_ms * 1e-3, device="cuda")
    total_ms = 1e3 * world * solves_per_step * args.steps / value  # the slowest rank's time
    if world > 1:
        dist.barrier()

    # ---- end to end through the host-buffer entry point
    e2e_times = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        both = eng.solve1d_arrays(stack, pts, M, 2)
        e2e_times.append(time.perf_counter() - t0)
    host = [{k: v[:P] for k, v in both.items()}, {k: v[P:] for k, v in both.items()}]
    e2e_value = replica_rate(world, solves_per_step, sum(e2e_times) / len(e2e_times), device="cuda")
    h2d = P * 16  # s and wavelength per point, once for both polarizations
    d2h = 2 * (P * n * (16 + 16 + 8 + 8) + P * 4 * 4)

    # ---- the plain path and the lossy variant (rank 0, after the timed region)
    line_extra = {}
    if rank == 0 and args.plain_points > 0:
        line_extra["plain"] = plain_rate(eng, stack, pts, args.plain_points, value)
    if rank == 0 and args.lossy_steps > 0:
        line_extra["lossy_c2"] = lossy_rate(eng, torch, est, flush, args, peak)
    if rank == 0 and args.serve_sample > 0:
        line_extra["serving"] = serving_sample(args)

    # ---- accuracy and CPU baseline (rank 0): the oracle on a bounded sample of the same points
    if rank == 0:
        threads = os.cpu_count() or 1
        sample_idx = np.linspace(0, P - 1, args.cpu_points).astype(int)
        rate, cpu_out, cpu_dt = cpu_rate(stack, pts[sample_idx], threads)
        err = 0.0
        for pol in (0, 1):
            for key in ("DEr", "DEt"):
                err = max(err, float(np.max(np.abs(host[pol][key][sample_idx] - cpu_out[pol][key]))))
        ok = all((host[pol]["status"] == 0).all() for pol in (0, 1))
        energy = max(float(np.max(np.abs(host[pol]["DEr"].sum(1) + host[pol]["DEt"].sum(1) - 1))) for pol in (0, 1))
        line_extra["cpu_baseline"] = {"value": rate, "unit": "solves/s", "cores": threads, "kind": "port",
                                      "sample": f"{len(sample_idx)} of the {P} points x TE+TM = {2 * len(sample_idx)} "
                                                f"solves, {cpu_dt:.1f} s wall"}
        line_extra["accuracy"] = {"max_abs_dDE_vs_oracle": err, "sample_solves": 2 * len(sample_idx),
                                  "all_status_ok": bool(ok), "max_energy_defect_all_points": energy}

    eig_avg_ms = eig_ms / max(1, eig_launches)
    # the grating's real permittivities take the Hermitian eigensolver unless it is switched off
    herm = not os.environ.get("RCWA_GB300_HERMITIAN", "").startswith("0")
    rot_per_matrix = rotations / (args.steps * 2 * P)  # the timed steps' TE and TM matrices
    reduced = os.environ.get("RCWA_GB300_SEAMS", "") != "reference"
    if herm:
        eig_flops_launch = P * herm_eig_flops(n, rot_per_matrix)
    else:
        eig_flops_launch = P * 105 * n ** 3
    total_flops = P * sum(engine_flops_per_solve(n, pol, rot_per_matrix, reduced) for pol in (0, 1))
    reference_flops = P * (flops_per_solve(n, 0) + flops_per_solve(n, 1))
    # the TE and TM eigensolves overlap in time: algorithmic flops of all of them over the time at least
    # one was running (union of their CUDA-event intervals on the two streams)
    achieved = eig_flops_launch * eig_launches / (eig_busy_ms * 1e-3) / 1e12
    step_ms = total_ms / args.steps
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64 (complex128)", "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD, "points": P, "M": M, "solves_per_step": solves_per_step,
                           "seed": SEED, **geo, "parallelism": f"replicas x{world}",
                           "l2": "flushed between steps (256 MB write); per-step device footprint is also > L2",
                           "eig_group": int(os.environ.get("RCWA_GB300_EIG_GROUP", "0") or 0)},
                "clocks": clocks,
                "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "gpu_launches": launches,
                "roofline": {"bound": "fp64", "kernel": (HERM_STAGE_KERNELS if herm else "eig_batch_kernel"),
                             "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                             "traffic": (HERM_STAGE_DRAM_BYTES_PER_MATRIX_N121 * P
                                         if herm and n == 121 and HERM_STAGE_DRAM_BYTES_PER_MATRIX_N121 else None),
                             "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of every launch of "
                                                "one eigensolve call per matrix (4096-matrix capture) x matrices per "
                                                "launch" if herm and n == 121 and HERM_STAGE_DRAM_BYTES_PER_MATRIX_N121
                                                else None),
                             "flops_model": (herm_flops_text(n, rot_per_matrix) if herm
                                             else "general QR: 105 n^3 per matrix"),
                             "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5",
                             "flops_per_launch": eig_flops_launch, "avg_launch_ms": eig_avg_ms,
                             "launches": eig_launches, "busy_ms": eig_busy_ms,
                             "timing": "TE and TM eigensolves run concurrently on two streams; achieved = "
                                       "their flops / busy time (union of launch intervals, CUDA events)"},
                "kernels_ms_per_step": {"eig": eig_ms / kstep, "lu": lu_ms / kstep, "gemm": gemm_ms / kstep,
                                        "eig_busy": eig_busy_ms / kstep,
                                        "note": f"summed launch durations of the two concurrent streams, from {kstep} "
                                                "instrumented steps run after the timed ones"},
                "step_fp64": {"algorithmic_tflop": total_flops / 1e12,
                              "achieved_tflops": total_flops / (step_ms * 1e-3) / 1e12,
                              "frac_of_peak": total_flops / (step_ms * 1e-3) / 1e12 / peak,
                              "model": "the engine's own operations (Hermitian eigensolve, reduced seams)",
                              "reference_sequence_tflop": reference_flops / 1e12,
                              "reference_sequence_rate_tflops": reference_flops / (step_ms * 1e-3) / 1e12},
                **line_extra}
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def plain_rate(eng, stack, pts, count, batched_value):
    """The plain path: `count` of the points, each solved alone through the host-buffer entry point, TE
    then TM (one solve per call), all FP64; solves/s and the batched value over it."""
    sel = pts[np.linspace(0, len(pts) - 1, count).astype(int)]
    eng.solve1d_arrays(stack, sel[:1], M, 0)  # warm
    t0 = time.perf_counter()
    for pol in (0, 1):
        for k in range(len(sel)):
            eng.solve1d_arrays(stack, sel[k:k + 1], M, pol)
    dt = time.perf_counter() - t0
    rate = 2 * len(sel) / dt
    return {"value": rate, "unit": "solves/s", "solves": 2 * len(sel), "seconds": dt,
            "batched_over_plain": batched_value / rate,
            "how": "one point and one polarization per call (rcwa_gpu_solve1d_batch with n_points = 1), host buffers"}


def lossy_rate(eng, torch, est, flush, args, peak):
    """The same headline sweep with an absorbing grating (n = 1.46 + 0.01i): the general Hessenberg + shifted
    complex QR eigensolver on every grating matrix. Device-resident points, CUDA events, L2 flushed;
    accuracy against the oracle on a sample."""
    from stablercwa_gb300.engine import launch_count
    stack, pts, geo = workload(n_points=args.points, ridge=LOSSY_RIDGE)
    n, P = 2 * M + 1, len(pts)
    d_pts = torch.tensor(pts, dtype=torch.float64, device="cuda")
    out = {"R": torch.empty((2 * P, n, 2), dtype=torch.float64, device="cuda"),
           "T": torch.empty((2 * P, n, 2), dtype=torch.float64, device="cuda"),
           "DEr": torch.empty((2 * P, n), dtype=torch.float64, device="cuda"),
           "DEt": torch.empty((2 * P, n), dtype=torch.float64, device="cuda"),
           "status": torch.empty(2 * P, dtype=torch.int32, device="cuda")}
    ptrs = {k: v.data_ptr() for k, v in out.items()}

    def step():
        eng.solve1d_device(stack, d_pts.data_ptr(), P, M, 2, ptrs)
    step()
    eng.synchronize()
    total = 0.0
    l0 = launch_count()
    for _ in range(args.lossy_steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(est)
        step()
        e1.record(est)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    launches = launch_count() - l0
    eng.set_kernel_timing(True)
    flush.fill_(1.0)
    torch.cuda.synchronize()
    step()
    eng.synchronize()
    eig_busy = eng.kernel_busy("eig")
    eig_ms, eig_launches = eng.kernel_time("eig")
    eng.set_kernel_timing(False)
    value = 2 * P * args.lossy_steps / (total * 1e-3)
    achieved = eig_launches * P * 105 * n ** 3 / (eig_busy * 1e-3) / 1e12 if eig_busy > 0 else None
    from oracle import oracle
    idx = np.linspace(0, P - 1, max(2, args.cpu_points // 4)).astype(int)
    host = {k: v.cpu().numpy() for k, v in out.items() if k in ("DEr", "DEt", "status")}
    err = 0.0
    for pol in (0, 1):
        ref = oracle.solve1d_batch(stack, pts[idx], M, pol, threads=os.cpu_count() or 1)
        for key in ("DEr", "DEt"):
            err = max(err, float(np.max(np.abs(host[key][pol * P + idx] - ref[key]))))
    return {"value": value, "unit": "solves/s", "steps": args.lossy_steps, "ms_per_step": total / args.lossy_steps,
            "gpu_launches": launches, "ridge_index": [LOSSY_RIDGE.real, LOSSY_RIDGE.imag],
            "eigensolver": "general: Hessenberg reduction + shifted complex QR + back substitution (eig_batch_kernel)",
            "eig_ms_per_step": eig_ms, "eig_busy_ms_per_step": eig_busy,
            "eig_roofline": {"achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                             "frac": achieved / peak if achieved else None, "flops_model": "105 n^3 per matrix"},
            "accuracy": {"max_abs_dDE_vs_oracle": err, "sample_solves": 2 * len(idx),
                         "all_status_ok": bool((host["status"] == 0).all())}}


# ------------------------------------------------------------------------------------- other configurations

CONICAL_POINTS, CONICAL_M = 1024, 40
CROSSED_POINTS, CROSSED_M = 256, 10


def workload_conical(seed=SEED):
    """Batched conical incidence, M = 40 (N = 81, 2N = 162): three gratings with 2-4 random
    segments (n 1.0..2.5, d 0.05..0.3) and one absorbing film n = 1.5+U(0,.5) + i U(0,.1), period
    0.574, nI 1.0, nII 1.46; 1024 points lambda 0.5..1.6, theta 0..60, phi 0..90 degrees."""
    from stablercwa_gb300 import Layer, Stack
    rng = np.random.default_rng(seed + 3)
    layers = []

    def grating():
        K = int(rng.integers(2, 5))
        inner = np.sort(rng.uniform(0.0, PERIOD, K - 1))
        return Layer.grating(rng.uniform(0.05, 0.3), [0.0, *inner, PERIOD], list(rng.uniform(1.0, 2.5, K)))
    layers += [grating(), grating()]
    layers.append(Layer.uniform(rng.uniform(0.05, 0.3), complex(1.5 + rng.uniform(0, 0.5), rng.uniform(0, 0.1))))
    layers.append(grating())
    stack = Stack(nI=1.0, nII=1.46, period=PERIOD, layers=layers)
    pts = np.stack([rng.uniform(0.5, 1.6, CONICAL_POINTS), rng.uniform(0.0, 60.0, CONICAL_POINTS),
                    rng.uniform(0.0, 90.0, CONICAL_POINTS)], axis=1)
    return stack, pts


def workload_crossed2d(seed=SEED):
    """Batched 2-D crossed grating, Mx = My = 10 (N = 441, 2N = 882): square lattice P 0.6..1.0,
    three patterned layers (d 0.05..0.3; a circular pillar r = 0.15..0.4 P staircased into 16 y strips
    or a w x h = 0.2..0.7 P rectangle, n = 2.0 in air) between five films (n 1.3..2.2, d 0.05..0.2),
    nI 1.0, nII 1.46; 256 points lambda 0.4..1.2 at normal incidence, s polarisation."""
    from stablercwa_gb300 import Layer2D, Stack2D, XProfile2D, jones_from_angles_2d
    rng = np.random.default_rng(seed + 4)
    P = rng.uniform(0.6, 1.0)

    def row(x0, x1):
        if x1 <= x0:
            return XProfile2D([0.0, P], [1.0])
        return XProfile2D([0.0, x0, x1, P], [1.0, 2.0, 1.0])

    def patterned():
        d = rng.uniform(0.05, 0.3)
        if rng.uniform() < 0.5:
            r = rng.uniform(0.15, 0.4) * P
            K = 16
            ye = [P * k / K for k in range(K + 1)]
            rows = []
            for k in range(K):
                yc = 0.5 * (ye[k] + ye[k + 1]) - 0.5 * P
                w = np.sqrt(max(r * r - yc * yc, 0.0))
                rows.append(row(0.5 * P - w, 0.5 * P + w))
            return Layer2D.patterned(d, ye, rows)
        w, h = rng.uniform(0.2, 0.7, 2) * P
        return Layer2D.patterned(d, [0.0, 0.5 * (P - h), 0.5 * (P + h), P],
                                 [row(0, 0), row(0.5 * (P - w), 0.5 * (P + w)), row(0, 0)])

    def film():
        return Layer2D.uniform(rng.uniform(0.05, 0.2), rng.uniform(1.3, 2.2))
    layers = [film(), patterned(), film(), patterned(), film(), patterned(), film(), film()]
    stack = Stack2D(nI=1.0, nII=1.46, layers=layers, Lx=P, Ly=P)
    es, ep = jones_from_angles_2d(90.0)
    pts = [(wl, 0.0, 0.0, es, ep) for wl in rng.uniform(0.4, 1.2, CROSSED_POINTS)]
    return stack, pts, {"period": float(P)}


def run_secondary(args):
    """--workload conical | crossed2d | plain: the conical and 2-D batched workloads, and the headline structure
    solved one point per call (the plain path). Measured through the host-buffer entry points (these
    paths take host arrays), so value and e2e are the same number."""
    import torch
    from stablercwa_gb300.engine import Engine, eig_rotations, launch_count
    eng = Engine()
    peak = fp64_peak_tflops(torch)
    herm_model = None  # (matrices per step, order) of the eigensolves that may take the Hermitian path
    if args.workload == "conical":
        stack, pts = workload_conical()
        n_eig_layers = sum(1 for L in stack.layers if not L.homogeneous)
        def step():
            return eng.solve_conical_arrays(stack, pts, CONICAL_M)
        solves = len(pts)
        eig_flops = solves * n_eig_layers * 2 * 105 * (2 * CONICAL_M + 1) ** 3
        herm_model = (solves * n_eig_layers * 2, 2 * CONICAL_M + 1)
        metric = "solves/s, batched conical sweep (M=40, 2N=162), full Jones per order"
        config = {"workload": workload_conical.__doc__.split(":")[0].strip(), "points": len(pts), "M": CONICAL_M,
                  "seed": SEED + 3}
    elif args.workload == "crossed2d":
        stack, pts, geo = workload_crossed2d()
        n_pat = sum(1 for L in stack.layers if not L.homogeneous)
        def step():
            return eng.solve2d_arrays(stack, pts, CROSSED_M, CROSSED_M)
        solves = len(pts)
        eig_flops = solves * n_pat * 105 * (2 * (2 * CROSSED_M + 1) ** 2) ** 3
        metric = "solves/s, batched 2-D solve2d sweep (Mx=My=10, N=441, 2N=882)"
        config = {"workload": "batched 2-D crossed grating, Mx=My=10 (N=441), 256 wavelengths", "points": len(pts), "M1": CROSSED_M, "M2": CROSSED_M,
                  "seed": SEED + 4, **geo}
    else:
        stack, all_pts, geo = workload()
        pts = all_pts[np.linspace(0, len(all_pts) - 1, 64).astype(int)]
        def step():
            return [eng.solve1d_arrays(stack, pts[k:k + 1], M, pol) for pol in (0, 1) for k in range(len(pts))]
        solves = 2 * len(pts)
        eig_flops = solves * 105 * (2 * M + 1) ** 3
        herm_model = (solves, 2 * M + 1)
        metric = "solves/s, plain path: the grating-on-mirror structure solved one point per call (M=60, N=121)"
        config = {"workload": "grating-on-mirror structure, 64 of its points x TE+TM, one solve per call", "M": M, "seed": SEED,
                  **geo}
    for _ in range(args.warmup):
        out = step()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    l0 = launch_count()
    eig_rotations()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = step()
        times.append(time.perf_counter() - t0)
    launches = launch_count() - l0
    rotations = eig_rotations()
    clocks = sampler.stop()
    # per-kernel-kind breakdown from one instrumented step after the timed ones (events around every
    # launch cost a little)
    eng.set_kernel_timing(True)
    step()
    roof_kernel, flops_model = "eig_batch_kernel", "general QR: 105 n^3 per matrix"
    if herm_model and not os.environ.get("RCWA_GB300_HERMITIAN", "").startswith("0"):
        # lossless layers: the Hermitian eigensolver; the model counts its matrices only (the few conical
        # Schur-basis eigensolves of order 2N inside the same timer are not counted)
        mats, order = herm_model
        rot = rotations / (mats * args.steps)
        eig_flops = mats * herm_eig_flops(order, rot)
        roof_kernel = HERM_STAGE_KERNELS
        flops_model = herm_flops_text(order, rot)
    eig_ms, _ = eng.kernel_time("eig")
    lu_ms, _ = eng.kernel_time("lu")
    gemm_ms, _ = eng.kernel_time("gemm")
    eng.set_kernel_timing(False)
    step_s = sum(times) / len(times)
    value = solves / step_s
    achieved = eig_flops / (eig_ms * 1e-3) / 1e12 if eig_ms > 0 else None
    line = {"metric": metric, "value": value, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (complex128)", "data": "synthetic (seeded)", "config": config,
            "clocks": clocks, "e2e": {"value": value, "unit": "solves/s", "note": "host-buffer entry point"},
            "gpu_launches": launches,
            "roofline": {"bound": "fp64", "kernel": roof_kernel, "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak if achieved else None, "flops_model": flops_model,
                         "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5"},
            "kernels_ms_per_step": {"eig": eig_ms, "lu": lu_ms, "gemm": gemm_ms,
                                    "other": 1e3 * step_s - (eig_ms + lu_ms + gemm_ms),
                                    "note": "one instrumented step run after the timed ones"}}
    if args.workload == "conical":
        from oracle import oracle
        threads = os.cpu_count() or 1
        idx = np.linspace(0, len(pts) - 1, args.cpu_points).astype(int)
        t0 = time.perf_counter()
        ref = oracle.solve_conical_batch(stack, pts[idx], CONICAL_M, threads=threads)
        dt = time.perf_counter() - t0
        err = max(float(np.nanmax(np.abs(out[k][idx] - ref[k]))) for k in ("DEr", "DEt"))
        line["cpu_baseline"] = {"value": len(idx) / dt, "unit": "solves/s", "cores": threads, "kind": "port",
                                "sample": f"{len(idx)} of the {len(pts)} points, {dt:.1f} s wall"}
        line["accuracy"] = {"max_abs_dDE_vs_oracle": err, "sample_solves": len(idx),
                            "all_status_ok": bool((out["status"] == 0).all())}
    elif args.workload == "crossed2d":
        line["accuracy"] = {"all_status_ok": bool((out["status"] == 0).all()),
                            "max_energy_defect": float(np.max(np.abs(out["DEr"].sum(1) + out["DEt"].sum(1) - 1.0)))}
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


# ------------------------------------------------------------------------------------- serving

def serve_requests(seed, count, repeat=1):
    """The serving mix: 70 % 1-D (M 20..150, 1..30 layers, each a grating with p 0.3 and at least one,
    K 2..5 random edges, n 1.0..2.5 + i 0..0.05, films likewise, period 0.5..1.5, lambda 0.4..1.6,
    theta 0..70, TE/TM), 20 % conical (M 20..60, built like the conical workload), 10 % 2-D (Mx = My 5..12,
    built like the 2-D workload). Returns (kind, stack, args) tuples. With repeat > 1 every drawn request is
    followed by repeat - 1 more of the same structure and truncation at new seeded points (a client
    scanning wavelengths and angles of one design)."""
    from stablercwa_gb300 import Layer, Stack
    rng = np.random.default_rng(seed)
    out = []
    for _ in range((count + repeat - 1) // repeat):
        u = rng.uniform()
        if u < 0.7:
            period = rng.uniform(0.5, 1.5)
            L = int(rng.integers(1, 31))
            is_grating = rng.uniform(size=L) < 0.3
            if not is_grating.any():
                is_grating[int(rng.integers(0, L))] = True
            layers = []
            for g in is_grating:
                d = rng.uniform(0.05, 0.3)
                if g:
                    K = int(rng.integers(2, 6))
                    inner = np.sort(rng.uniform(0.0, period, K - 1))
                    vals = [complex(rng.uniform(1.0, 2.5), rng.uniform(0.0, 0.05)) for _ in range(K)]
                    layers.append(Layer.grating(d, [0.0, *inner, period], vals))
                else:
                    layers.append(Layer.uniform(d, complex(rng.uniform(1.0, 2.5), rng.uniform(0.0, 0.05))))
            stack = Stack(nI=1.0, nII=1.46, period=period, layers=layers)
            out.append(("1d", stack, dict(wavelength=rng.uniform(0.4, 1.6), theta=rng.uniform(0.0, 70.0),
                                          M=int(rng.integers(20, 151)), pol=int(rng.integers(0, 2)))))
        elif u < 0.9:
            stack, _ = workload_conical(int(rng.integers(0, 1 << 30)))
            out.append(("conical", stack, dict(wavelength=rng.uniform(0.5, 1.6), theta=rng.uniform(0.0, 60.0),
                                               phi=rng.uniform(0.0, 90.0), M=int(rng.integers(20, 61)))))
        else:
            stack, pts, _ = workload_crossed2d(int(rng.integers(0, 1 << 30)))
            Mx = int(rng.integers(5, 13))
            out.append(("2d", stack, dict(wavelength=rng.uniform(0.4, 1.2), M1=Mx, M2=Mx, jones=(pts[0][3], pts[0][4]))))
        kind, stack, a = out[-1]
        for _ in range(repeat - 1):  # the same design at other points
            b = dict(a)
            b["wavelength"] = a["wavelength"] * rng.uniform(0.9, 1.1)
            if "theta" in b:
                b["theta"] = min(70.0, a["theta"] + rng.uniform(0.0, 5.0))
            out.append((kind, stack, b))
    return out[:count]


def serve_submit(srv, req):
    kind, stack, a = req
    if kind == "1d":
        return srv.submit_1d(stack, a["wavelength"], a["theta"], a["M"], a["pol"])
    if kind == "conical":
        return srv.submit_conical(stack, a["wavelength"], a["theta"], a["phi"], a["M"])
    return srv.submit_2d(stack, a["wavelength"], 0.0, 0.0, a["M1"], a["M2"], a["jones"])


def serve_run(reqs, slots, rate=None, seed=0, max_batch=0):
    """Submit reqs (all at once, or with Poisson arrivals at `rate` per second) to a server with
    `slots` worker slots; returns (makespan s, latencies s, per-kind latencies, statuses)."""
    from stablercwa_gb300.engine import Server
    srv = Server(slots=slots, max_batch=max_batch)
    rng = np.random.default_rng(seed)
    arrivals = np.zeros(len(reqs)) if rate is None else np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    t0 = time.perf_counter()
    tickets = []
    for req, at in zip(reqs, arrivals):
        delay = at - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets.append(serve_submit(srv, req))
    done = [srv.wait(t) for t in tickets]
    srv.close()
    first = min(i["submit_s"] for i, _ in done)
    makespan = max(i["finish_s"] for i, _ in done) - first
    lat = np.array([i["finish_s"] - i["submit_s"] for i, _ in done])
    kinds = {}
    for (kind, _, _), l in zip(reqs, lat):
        kinds.setdefault(kind, []).append(l)
    ok = all(i["code"] == 0 and int(r["status"]) == 0 for i, r in done)
    return makespan, lat, kinds, ok


def serving_sample(args):
    """A bounded sample of the serving mix for the headline line: its first `serve_sample` requests
    submitted at once to the serving loop (served solves/s, p50 / p99 of completion - submission), then
    the same requests one at a time on one slot (the plain one-request-per-launch path)."""
    reqs = serve_requests(SEED + 5, args.serve_sample)
    mk, lat, kinds, ok = serve_run(reqs, args.serve_slots)
    mk1, lat1, _, ok1 = serve_run(reqs, 1, max_batch=1)
    return {"value": len(reqs) / mk, "unit": "solves/s", "requests": len(reqs),
            "kinds": {k: len(v) for k, v in kinds.items()}, "slots": args.serve_slots,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)), "makespan_s": mk,
            "plain_one_slot": {"value": len(reqs) / mk1, "makespan_s": mk1, "p50_s": float(np.percentile(lat1, 50)),
                               "p99_s": float(np.percentile(lat1, 99))},
            "served_over_plain": mk1 / mk, "all_ok": bool(ok and ok1),
            "how": "the first requests of the seeded serving mix (70 % 1-D, 20 % conical, 10 % 2-D), all submitted "
                   "at once; the full mix with Poisson arrivals is --workload serve"}


def run_serve(args):
    reqs = serve_requests(SEED + 5, args.serve_requests)
    stats = {}

    def summary(lat):
        return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "mean_s": float(np.mean(lat))}
    makespan, lat, kinds, ok = serve_run(reqs, args.serve_slots)
    capacity = len(reqs) / makespan
    stats["saturated"] = {"solves_per_s": capacity, "makespan_s": makespan, **summary(lat), "all_ok": ok,
                          "by_kind": {k: {**summary(np.array(v)), "count": len(v)} for k, v in kinds.items()}}
    for frac in args.serve_rates:
        mk, lat, kinds, ok = serve_run(reqs, args.serve_slots, rate=frac * capacity, seed=SEED + 6)
        stats[f"poisson_{frac:g}x"] = {"offered_per_s": frac * capacity, "solves_per_s": len(reqs) / mk, **summary(lat),
                                        "all_ok": ok,
                                        "by_kind": {k: {**summary(np.array(v)), "count": len(v)} for k, v in kinds.items()}}
    mk, lat, kinds, ok = serve_run(reqs, 1, max_batch=1)
    stats["plain_one_slot"] = {"solves_per_s": len(reqs) / mk, "makespan_s": mk, **summary(lat), "all_ok": ok,
                               "by_kind": {k: {**summary(np.array(v)), "count": len(v)} for k, v in kinds.items()}}
    if args.serve_repeat > 1:
        # the same mix where each design is requested at several points: same-structure requests share calls
        rreqs = serve_requests(SEED + 5, args.serve_requests, args.serve_repeat)
        mk, lat, kinds, ok = serve_run(rreqs, args.serve_slots)
        mk1, lat1, _, ok1 = serve_run(rreqs, 1, max_batch=1)
        stats[f"repeat_{args.serve_repeat}"] = {
            "solves_per_s": len(rreqs) / mk, "makespan_s": mk, **summary(lat), "all_ok": ok and ok1,
            "plain_one_slot_solves_per_s": len(rreqs) / mk1, "served_over_plain": mk1 / mk,
            "by_kind": {k: {**summary(np.array(v)), "count": len(v)} for k, v in kinds.items()}}
    head = stats.get("poisson_1x", stats["saturated"])
    line = {"metric": "served solves/s and p50/p99 latency, mixed 1-D / conical / 2-D requests (70/20/10)",
            "value": head["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f64 (complex128)", "data": "synthetic (seeded)",
            "config": {"workload": "serving mix", "requests": len(reqs), "slots": args.serve_slots, "seed": SEED + 5},
            "p50_s": head["p50_s"], "p99_s": head["p99_s"],
            "vs_plain": head["solves_per_s"] / stats["plain_one_slot"]["solves_per_s"], "runs": stats}
    print(json.dumps(line), flush=True)
    return 0


def run_eig_only(n, batch, group, hermitian=False):
    """Profiling case for the eigensolver alone: `batch` layer matrices of order n in the benchmark's
    form (Toeplitz of a binary grating, index 1.46+0.01i, fill 0.4, plus Kx^2 with sin(theta) in
    0.75..0.95, lambda/period 0.61), eigensolved twice on device by the general solver; with
    `hermitian`, the lossless index 1.46 and the Hermitian solver."""
    import torch
    from stablercwa_gb300.engine import Engine
    if group:
        os.environ["RCWA_GB300_EIG_GROUP"] = str(group)
    rng = np.random.default_rng(1)
    M = n // 2
    h = np.subtract.outer(np.arange(n), np.arange(n))
    e1 = complex(1.46, 0.0 if hermitian else 0.01) ** 2
    with np.errstate(invalid="ignore", divide="ignore"):
        eps = np.where(h == 0, 0.4 * e1 + 0.6, (e1 - 1) * np.sin(np.pi * h * 0.4) / (np.pi * h))
    mats = []
    for _ in range(32):
        kx = rng.uniform(0.75, 0.95) + (np.arange(n) - M) * 0.61
        mats.append((-eps + np.diag(kx * kx)).astype(np.complex128))
    A = np.ascontiguousarray(np.array(mats)[np.arange(batch) % 32].transpose(0, 2, 1)).astype(np.complex128)
    dA = torch.tensor(A.view(np.float64), device="cuda")
    assert dA.numel() * 8 == batch * n * n * 16
    dW = torch.empty((batch, n, 2), dtype=torch.float64, device="cuda")
    dV = torch.empty((batch, n, n, 2), dtype=torch.float64, device="cuda")
    dI = torch.empty(batch, dtype=torch.int32, device="cuda")
    eng = Engine()
    est = torch.cuda.ExternalStream(eng.stream())
    ms = []
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(est)
        if hermitian:
            eng.eig_hermitian_batch_device(n, batch, dA.data_ptr(), dW.data_ptr(), dV.data_ptr(), dI.data_ptr())
        else:
            eng.eig_batch_device(n, batch, dA.data_ptr(), dW.data_ptr(), dV.data_ptr(), dI.data_ptr())
        e1.record(est)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    bad = int((dI != 0).sum().item())
    print(json.dumps({"eig_only": {"n": n, "batch": batch, "group": group, "hermitian": hermitian,
                                   "not_converged": bad, "ms_second_call": ms[1]}}))
    return 0 if bad == 0 else 1


def run_gemm_only(batch, m, k, n):
    """Profiling case for the complex product alone: `batch` products of seeded normal complex m x k and
    k x n matrices through rcwa_gpu_multiply_batch (the tensor-core path unless RCWA_GB300_GEMM=fp64),
    three times; the device time of the third (digit splits + product kernel, CUDA events on the engine's
    stream) and its FP64-equivalent rate 8 m n k / time."""
    from stablercwa_gb300.engine import Engine
    rng = np.random.default_rng(2)
    a = rng.normal(size=(batch, m, k)) + 1j * rng.normal(size=(batch, m, k))
    b = rng.normal(size=(batch, k, n)) + 1j * rng.normal(size=(batch, k, n))
    eng = Engine()
    eng.multiply_batch(a, b)
    eng.set_kernel_timing(True)
    ms = []
    for _ in range(2):
        eng.kernel_time("gemm")
        c = eng.multiply_batch(a, b)
        ms.append(eng.kernel_time("gemm")[0])
    eng.set_kernel_timing(False)
    eng.close()
    err = float(np.max(np.abs(c[:2] - a[:2] @ b[:2])))
    print(json.dumps({"gemm_only": {"batch": batch, "m": m, "k": k, "n": n, "ms": ms[-1],
                                    "tflops_fp64_equivalent": 8.0 * batch * m * n * k / (ms[-1] * 1e-3) / 1e12,
                                    "max_abs_err_first_two": err}}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--eig-group", type=int, default=0)
    ap.add_argument("--cpu-points", type=int, default=128)
    ap.add_argument("--points", type=int, default=N_POINTS,
                    help="sweep points per step (the headline is 4096; fewer only for small profiling captures)")
    ap.add_argument("--ref-points", type=int, default=128)
    ap.add_argument("--plain-points", type=int, default=32,
                    help="points of the plain one-solve-per-call line in the headline run (0: skip)")
    ap.add_argument("--lossy-steps", type=int, default=1,
                    help="timed steps of the absorbing-grating sweep line in the headline run (0: skip)")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-slots", type=int, default=48)
    ap.add_argument("--serve-repeat", type=int, default=8,
                    help="--workload serve: also run the mix with each design requested at this many points (1: skip)")
    ap.add_argument("--serve-sample", type=int, default=40,
                    help="requests of the serving mix run in the headline line (0: skip)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[0.5, 1.0])
    ap.add_argument("--workload", choices=["sweep", "conical", "crossed2d", "plain", "serve"], default="sweep",
                    help="sweep (default, the headline line), conical, crossed2d (2-D), plain one-point-per-call, "
                         "serve (the serving mix)")
    ap.add_argument("--hermitian", action="store_true", help="--eig-only: lossless matrices, Hermitian solver")
    ap.add_argument("--eig-only", nargs=2, type=int, metavar=("N", "BATCH"), default=None,
                    help="profiling case: the eigensolver alone on BATCH layer matrices of order N")
    ap.add_argument("--gemm-only", nargs=4, type=int, metavar=("BATCH", "M", "K", "N"), default=None,
                    help="profiling case: BATCH complex products of m x k by k x n, digit splits and product kernel")
    args = ap.parse_args()
    if args.gemm_only:
        return run_gemm_only(*args.gemm_only)
    if args.eig_only:
        return run_eig_only(args.eig_only[0], args.eig_only[1], args.eig_group, args.hermitian)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload != "sweep":
        return run_secondary(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
