"""Benchmark: batched hybrid inverse of the ADRT at N=256 on one GB300 (replicas across GPUs).

Workload (one step): the hybrid explicit inverse (fastops.FastHybrid.apply semantics) of a batch of 64 noisy
sinograms of seeded 10-ellipse phantoms at N = 256 (n = 8), inner degrees capped at p = 32, dense low-frequency
table for d_k > 16, FP32 row engine / FFTs and cross-quadrant preconditioner (--stencil ff|fp64 for the FP64-class
forms) with FP64 tables; the outer iteration's state is float-float (FP32 hi/lo planes, about 48 bits) with the FP32
stencil and FP64 with the others. Metric: whole-job reconstructions per second. Every step's inputs
(268 MB of FP64 sinograms) exceed the 129 MB L2, so no flush is needed between steps.

  value : device-resident sinograms, K timed replays of the captured apply (CUDA events, barrier + sync both sides);
          an instrumented eager pass before it gives the per-kernel timings, the launch count and `eager`.
  e2e   : the public API FastHybridGpu.apply on pinned host sinograms into a pinned host result every step (H2D + D2H
          inside the timed region; consecutive calls overlap a batch's copy with the previous batch's graph).
  roofline : the row engine (rows_prog_kernel), the dominant kernel, timed live with CUDA events on its stream;
          algorithmic FLOPs = level-rows x 8N (the reference's cost unit, fastops.py:166); peak = FP32 FMA
          throughput measured in this run by the library's probe kernel.
  cpu_baseline : the reference's C++-engine path (FastHybridCpp semantics: C row kernels + NumPy) timed on this
          host's cores on one image of the same workload, same plan.
  extras (one-GPU runs, --no-extras to skip): preconditioner_ff / _fp32 (the other preconditioner precision),
          adrt_int32, cgls, serve (p50/p99 at a sustainable rate and at 2000 req/s), uneven (stream-per-class graph
          and persistent rows), large (N=2048, batch 1 and 8).
`--impl reference` times only that CPU path (rank 0) on the same config and prints its own line; --mode
serve|uneven|large|adrt runs one of the other workloads alone.
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

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_LOG2, BATCH, P_CAP, DENSE_CAP, REL_SIGMA = 8, 64, 32, 16, 1e-3
STENCIL = "fp32"  # the cross-quadrant preconditioner in FP32; the FP64-class (float-float) run is reported beside it
METRIC = "hybrid-inverse recon/s at N=256 (<=1e-5 vs FP64)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--n", type=int, default=N_LOG2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-region", action="store_true", help="cudaProfilerStart/Stop around the timed steps")
    ap.add_argument("--mode", default="batch", choices=["batch", "serve", "uneven", "large", "adrt"],
                    help="batch: the headline N=256 batch-64 workload; serve: Poisson mixed-N request loop; "
                         "uneven: 512 mixed N/p/method sinograms in one CUDA graph; large: N=2048, batch 1 and 8")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--stencil", default=STENCIL, choices=["fp32", "ff", "fp64"],
                    help="precision of the cross-quadrant preconditioner (ff: float-float, about 48 bits)")
    ap.add_argument("--high-rows", default="dense", choices=["dense", "ff"],
                    help="large mode: the rows with d_k > dense_cap as dense operators or compensated rows")
    ap.add_argument("--no-extras", action="store_true",
                    help="batch mode: skip the short serve / uneven / large runs appended to the line")
    return ap.parse_args()


STENCIL_NAMES = {"fp32": "fp32", "ff": "float-float (fp64-class)", "fp64": "fp64"}


def config(args, world):
    N = 1 << args.n
    return {"workload": f"hybrid inverse, N={N}, batch {args.batch} per GPU, p={P_CAP}, dense_cap={DENSE_CAP}, "
                        f"10-ellipse phantoms + noise {REL_SIGMA:g} max|b|",
            "N": N, "global_batch": args.batch * world, "p": P_CAP, "dense_cap": DENSE_CAP, "method": "hybrid",
            "precond": "g1",
            "precision": f"fp32 rows/FFT, cross-quadrant inverse {STENCIL_NAMES[getattr(args, 'stencil', STENCIL)]}, "
                         "fp64 tables, outer state "
                         + ("float-float (fp32 hi/lo planes)" if getattr(args, "stencil", STENCIL) == "fp32" else "fp64"),
            "parallelism": f"replicas x{world}", "l2": "inputs (268 MB/step) larger than L2; no flush"}


def sinograms(pkg, n, B, seed0, device):
    """Seeded phantoms -> ADRT on the GPU (FP64) -> i.i.d. noise sigma = 1e-3 max|b| (per sinogram)."""
    import torch

    N = 1 << n
    xs = np.stack([pkg.phantoms.ellipse_phantom(N, seed=seed0 + i) for i in range(B)])
    b = pkg.adrtcore.adrt(n, torch.from_numpy(xs).to(device))
    g = torch.Generator(device=device).manual_seed(seed0)
    noise = torch.randn(b.shape, generator=g, device=device, dtype=b.dtype)
    return b + REL_SIGMA * b.abs().amax(dim=(1, 2, 3), keepdim=True) * noise


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx, self.rows, self.proc = str(gpu_index), [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", self.idx], stdout=subprocess.PIPE, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def fp32_peak(pkg, torch):
    """FP32 FLOP/s of the library's FMA probe kernel (8 independent chains per thread, all SMs)."""
    C = pkg._lib
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4000
    out = torch.empty(blocks * threads, dtype=torch.float32, device="cuda")
    st = C.stream_handle()
    for _ in range(2):
        C.call("adrt_fp32_probe", blocks, threads, 200, C.ptr(out), st)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(3):
        e0.record()
        C.call("adrt_fp32_probe", blocks, threads, iters, C.ptr(out), st)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, blocks * threads * iters * 128 / (e0.elapsed_time(e1) * 1e-3))
    return best


def cpu_reference_time(n, plan_kw, b_one, reps, threads):
    """Seconds per apply of the reference's C++-engine path on the host (oracle/_ref when built, else the port)."""
    from oracle import cpu_engine as CE

    H = CE.hybrid_cpu(n, plan_kw, threads=threads)
    H.apply(b_one)  # warm-up (and the dense tables)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        H.apply(b_one)
        ts.append(time.perf_counter() - t0)
    return min(ts), H.eng.kind


def traffic_per_launch():
    """DRAM bytes per launch of the row kernel from the committed ncu summary (null when not captured)."""
    path = os.path.join(REPO, "profiles", "rows_prog_kernel_hybrid_n8_b64_dram.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def run_reference(args):
    """CPU reference arm: the reference's C++ row kernels + NumPy glue on the host cores, same workload."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    import __graft_entry__ as ge

    pkg = ge.load_package()
    from oracle import adrt_np as A
    from oracle import cpu_engine as CE
    from oracle import oblique_np as O

    n, N = args.n, 1 << args.n
    threads = os.cpu_count() or 1
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    CE.build()
    # the reference's own setup on the CPU: power iteration (fastcpp conventions), degrees capped at p, Lanczos
    lam = O.power_lam_max(n, O.offset_z(2 * N), 2, seeds=(0, 1))
    H = CE.hybrid_cpu(n, dict(lam_max=lam, deg_cap=P_CAP, dense_cap=DENSE_CAP, outer=(1.0, 2.0, 3)), threads=threads)
    G1 = O.G1_apply
    lo, hi, D = O.outer_interval(N, H.Gh, G1, H.P, 1e-10)
    H.lo, H.hi, H.outer_deg = lo, hi, D
    x = pkg.phantoms.ellipse_phantom(N, seed=0)
    b = pkg.phantoms.add_noise(A.adrt(n, x), REL_SIGMA, seed=1)
    for _ in range(args.warmup):
        H.apply(b)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        H.apply(b)
    dt = (time.perf_counter() - t0) / args.steps
    v = 1.0 / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "recon/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, world),
            "cpu_baseline": {"value": v, "unit": "recon/s", "cores": threads, "kind": H.eng.kind,
                             "sample": f"one N={N} sinogram per step (the batch's first), same plan"},
            "e2e": {"value": v, "unit": "recon/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measured_hbm_peak():
    """The machine's measured copy bandwidth (GB/s) from MEASURED_PEAKS.json beside this file, else the fallback."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def hbm_rooflines(ktimer, pipe):
    """Achieved HBM GB/s of the offset-FFT kernels in the timed region (CUDA events on their stream) against the
    measured copy bandwidth; algorithmic bytes per launch: the image read (the FP32 hi plane of a float-float outer
    state, else the FP64 image) and the packed rows (complex64) written by the image pack, the packed rows read and
    the three FP32 partial images written by the unpack."""
    N, B = pipe.plan.N, pipe.B
    isz = pipe.real.itemsize
    y_bytes = B * (4 * N) * N * 2 * isz  # packed rows: 2L = 4N rows of N complex per image
    img_bytes = 4 if getattr(pipe, "ff_state", False) else 8
    bytes_ = {"pack_fft_kernel (image)": B * N * N * img_bytes + y_bytes,
              "ifft_unpack_kernel": y_bytes + 3 * B * N * N * isz}
    names = {"pack_image": "pack_fft_kernel (image)", "unpack": "ifft_unpack_kernel"}
    peak, src = measured_hbm_peak()
    out = {}
    for key, label in names.items():
        ms = [a.elapsed_time(b) for n, a, b in ktimer if n == key]
        if ms:
            gbs = bytes_[label] / (float(np.mean(ms)) * 1e-3) / 1e9
            out[label] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                          "bytes_per_launch": bytes_[label], "launch_us": float(np.mean(ms)) * 1e3}
    return {"kernels": out, "peak_source": src}


def max_over_ranks(x, world, device):
    """The slowest rank's time (replicas: the job ends when the last rank ends); a no-op for one process."""
    import torch
    import torch.distributed as dist

    if world <= 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(batch_per_rank, world, seconds):
    """Whole-job reconstructions/s of `world` replicas, each inverting `batch_per_rank` images in `seconds`."""
    return batch_per_rank * world / seconds


def single_image_rates(H, b_dev, steps, torch):
    """Reconstructions/s of one sinogram at a time on the device: eager Pipeline.apply at batch 1 (the plain
    single-image GPU path) and the same apply replayed from a CUDA graph."""
    pipe = H.pipeline(1)
    b1 = b_dev[:1].contiguous()
    for _ in range(3):
        pipe.apply(b1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        pipe.apply(b_dev[i % b_dev.shape[0]:][:1])
    torch.cuda.synchronize()
    eager = steps / (time.perf_counter() - t0)
    pipe.capture()
    for _ in range(3):
        pipe.replay(b1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(steps):
        pipe.replay(b_dev[i % b_dev.shape[0]:][:1])
    torch.cuda.synchronize()
    graph = steps / (time.perf_counter() - t0)
    return {"eager_recon_s": eager, "graph_recon_s": graph, "unit": "recon/s",
            "how": f"{steps} single sinograms, device-resident, host clock around the loop"}


def run_ours(args):
    import torch
    import torch.distributed as dist

    import __graft_entry__ as ge

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    pkg = ge.load_package()
    C = pkg._lib
    n, N, B = args.n, 1 << args.n, args.batch

    H = pkg.FastHybridGpu(n, deg_cap=P_CAP, dense_cap=DENSE_CAP, precision="fp32", device=dev,
                          stencil_precision=args.stencil)
    b_dev = sinograms(pkg, n, B, seed0=1000 * rank, device=dev)
    pipe = H.pipeline(B)

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- device-resident throughput
    for _ in range(args.warmup):
        pipe.apply(b_dev)
    torch.cuda.synchronize()
    timer = []
    pipe.tables.timer = timer
    ktimer = []
    pipe.timer = ktimer
    barrier()
    torch.cuda.synchronize()
    l0 = C.load().adrt_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if args.profile_region:
        torch.cuda.profiler.start()
    e0.record()
    for _ in range(args.steps):
        pipe.apply(b_dev)
    e1.record()
    torch.cuda.synchronize()
    if args.profile_region:
        torch.cuda.profiler.stop()
    barrier()
    launches = (C.load().adrt_launch_count() - l0) // args.steps
    pipe.tables.timer = None
    pipe.timer = None
    ms_eager = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    # the value: the same applies replayed from the captured CUDA graph (the input already in the graph's input
    # buffer on the device), so the step carries no host launch gaps; the instrumented eager pass above gives the
    # per-kernel timings and the launch count
    pipe.capture()
    pipe.b_in.copy_(b_dev)
    for _ in range(args.warmup):
        pipe.replay()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        time.sleep(0.3)
        e0.record()
        for _ in range(args.steps):
            pipe.replay()
        e1.record()
        torch.cuda.synchronize()
    barrier()
    pipe.tables.raise_if_error()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value = replica_throughput(B, world, ms * 1e-3)
    # the G_h launches of the polynomial rows (one per outer step): mean duration and algorithmic FLOPs
    from adrt_pinv_gb300.device import fuse_ops

    g_ms = [a.elapsed_time(b) for a, b, ops in timer if ops == fuse_ops(pipe.ops["G"])]
    rows_launch_ms = float(np.mean(g_ms)) if g_ms else None
    flops_per_launch = pipe.tables.main_level_rows(pipe.ops["G"]) * B * 8 * N

    # ---- end to end through the public API with pinned host buffers
    b_host = torch.empty(b_dev.shape, dtype=b_dev.dtype, pin_memory=True)
    b_host.copy_(b_dev)
    out_host = torch.empty((B, N, N), dtype=torch.float64, pin_memory=True)
    for _ in range(2):
        H.apply(b_host, out=out_host)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        H.apply(b_host, out=out_host)
    H.check()  # waits for the last call and checks its dense kernel's error flag
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    barrier()
    e2e_value = replica_throughput(B, world, max_over_ranks(e2e_s, world, dev))

    # ---- the plain single-image GPU path (batch 1, eager launches) and the same under a CUDA graph
    single = single_image_rates(H, b_dev, args.steps, torch)
    barrier()

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # ---- accuracy of this run against the FP64 CPU reference path on one image (same plan)
    peak = fp32_peak(pkg, torch)
    line = {"metric": METRIC, "value": value, "unit": "recon/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipse phantoms + Gaussian noise)",
            "config": config(args, world), "gpu_launches": int(launches),
            "eager": {"value": replica_throughput(B, world, ms_eager * 1e-3), "ms_per_step": ms_eager,
                      "how": "the same steps launched eagerly from Python (instrumented for the kernel timings)"},
            "clocks": clk.summary(),
            "single_image": single, "batched_over_single_image": value / world / single["eager_recon_s"],
            "e2e": {"value": e2e_value, "unit": "recon/s", "h2d_bytes_per_step": int(b_host.numel() * 8),
                    "d2h_bytes_per_step": int(out_host.numel() * 8)}}
    line["roofline_hbm"] = hbm_rooflines(ktimer, pipe)
    if rows_launch_ms:
        achieved = flops_per_launch / (rows_launch_ms * 1e-3) / 1e12
        tr = traffic_per_launch()  # captured at N=256, batch 64; rows scale with the batch
        tr = tr * B / 64 if tr is not None and n == 8 else None
        line["roofline"] = {"bound": "fp32", "kernel": "rows_prog_kernel (G_h op list, polynomial rows)",
                            "achieved": achieved, "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved * 1e12 / peak,
                            "peak_source": "measured in this run: FP32 FMA probe kernel",
                            "flop_per_launch": flops_per_launch, "launch_ms": rows_launch_ms,
                            "traffic": tr, "traffic_unit": "bytes/launch (ncu dram read+write)",
                            "traffic_source": ("not measured in this run: the committed ncu capture "
                                               "profiles/rows_prog_kernel_hybrid_n8_b64_dram.txt (N=256, batch 64), "
                                               "scaled by batch/64" if tr is not None else None)}
    if not args.no_cpu_baseline:
        plan_kw = dict(lam_max=H.plan.lam_max, deg=H.deg, dense_cap=DENSE_CAP, outer=(H.lo, H.hi, H.outer_deg))
        b_one = b_dev[0].cpu().numpy()
        threads = os.cpu_count() or 1
        t_cpu, kind = cpu_reference_time(n, plan_kw, b_one, 2, threads)
        from oracle import cpu_engine as CE

        ref = CE.hybrid_cpu(n, plan_kw, threads=threads).apply(b_one)
        got = H.apply(b_dev[:1])[0].cpu().numpy()
        line["rel_err_vs_fp64"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        line["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "recon/s", "cores": threads, "kind": kind,
                                "sample": f"one N={N} sinogram of the batch, min of 2 applies after a warm-up"}
    else:
        ref = None
    if world == 1 and not args.no_extras:
        other = "ff" if args.stencil != "ff" else "fp32"
        line[f"preconditioner_{other}"] = stencil_variant(pkg, H, b_dev, args.steps, other, ref, torch)
        line["adrt_int32"] = adrt_int32_timing(pkg, n, B, args.steps, torch)
        line["cgls"] = cgls_timing(pkg, n, 16, 50, torch)
        line.update(extras(pkg, dev, args))
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def adrt_int32_timing(pkg, n, B, steps, torch):
    """The spatial ADRT forward and transpose on B int32 images with values in [0, 255] (bit-exact integer sums),
    each timed with CUDA events; HBM roofline per call from the bytes every level pass moves (level m reads the
    level-(m-1) data and writes level m; the transpose mirrors it; the first forward level reads the image, the last
    transpose level writes it), against the measured copy bandwidth; checked bit-exact against the oracle on one
    image."""
    from oracle import adrt_np as A

    N = 1 << n
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(5)
    x = torch.randint(0, 256, (B, N, N), dtype=torch.int32, device=dev, generator=g)
    b = torch.empty((B, 4, 2 * N - 1, N), dtype=torch.int32, device=dev)
    xt = torch.empty_like(x)
    scratch = torch.empty(2 * B * 4 * (2 * N - 1) * N, dtype=torch.int32, device=dev)
    C = pkg._lib
    st = C.stream_handle()

    def fwd():
        C.call("adrt_forward", C.I32, n, B, C.ptr(x), C.ptr(b), C.ptr(scratch), st)

    def adj():
        C.call("adrt_transpose", C.I32, n, B, C.ptr(b), C.ptr(xt), C.ptr(scratch), st)

    lvl = lambda m: 4 * (N + (1 << m) - 1) * N * 4  # bytes of level-m data, four quadrants, int32
    fwd_bytes = B * (N * N * 4 + sum(lvl(m) for m in range(1, n + 1)) + sum(lvl(m) for m in range(1, n)))
    peak, _ = measured_hbm_peak()
    out = {}
    for name, fn in (("forward", fwd), ("transpose", adj)):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        gbs = fwd_bytes / (ms * 1e-3) / 1e9
        out[name] = {"ms": ms, "images_per_s": B / (ms * 1e-3), "bytes_per_call": fwd_bytes, "achieved_gbs": gbs,
                     "peak_gbs": peak, "frac": gbs / peak}
    x0 = x[0].cpu().numpy()
    out["bit_exact_forward"] = bool(np.array_equal(b[0].cpu().numpy(), A.adrt(n, x0, dtype=np.int64)))
    out["bit_exact_transpose"] = bool(np.array_equal(xt[0].cpu().numpy(),
                                                     A.adrt_T(n, b[0].cpu().numpy(), dtype=np.int64)))
    out["workload"] = f"{B} int32 images N={N}, values U[0,255]"
    return out


def cgls_timing(pkg, n, B, iters, torch):
    """CGLS (pinv.py:23-48) on B noisy phantom sinograms at N = 2^n for a fixed number of iterations (tol = 0, so
    no image stops): iterations per second and the HBM rate of an iteration, counting per image the spatial ADRT
    and its transpose in FP64 (every level pass reads its input and writes its output) plus the vector passes (two
    inner products, the x/r update and the direction update)."""
    from adrt_pinv_gb300 import pinv

    N = 1 << n
    dev = torch.device("cuda")
    b = _phantom_sinos(pkg, n, B, 4242, dev, REL_SIGMA)
    S = pinv.CglsSolver(n, B, maxit=iters + 2, tol=0.0, device=dev, block=iters)
    S.start(b)
    S.iterate(2)  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    S.iterate(iters)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    lvl = lambda m: 4 * (N + (1 << m) - 1) * N * 8
    adrt_bytes = N * N * 8 + sum(lvl(m) for m in range(1, n + 1)) + sum(lvl(m) for m in range(1, n))
    sino, img = 4 * (2 * N - 1) * N * 8, N * N * 8
    vec_bytes = sino + img + (2 * img + 2 * sino) + (2 * img + img) + img  # <q,q>, <s,s>, x/r update, p update
    per_iter = B * (2 * adrt_bytes + vec_bytes)
    peak, _ = measured_hbm_peak()
    gbs = per_iter / (ms * 1e-3) / 1e9
    its = int(S.it[0].item())
    return {"workload": f"CGLS on {B} sinograms N={N}, {iters} iterations (tol 0), FP64",
            "ms_per_iteration": ms, "image_iterations_per_s": B / (ms * 1e-3), "bytes_per_iteration": per_iter,
            "achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak, "iterations_run": its}


def stencil_variant(pkg, H, b_dev, steps, stencil, ref, torch):
    """The same batch with the cross-quadrant preconditioner in another precision (ff: float-float, FP64-class):
    throughput (device-resident, CUDA events) and the first image's error against the CPU reference path."""
    from adrt_pinv_gb300.device import Pipeline

    pipe = Pipeline(H.plan, b_dev.shape[0], "fp32", b_dev.device, stencil)
    for _ in range(3):
        pipe.apply(b_dev)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        x = pipe.apply(b_dev)
    e1.record()
    torch.cuda.synchronize()
    pipe.tables.raise_if_error()
    ms = e0.elapsed_time(e1) / steps
    out = {"value": b_dev.shape[0] / (ms * 1e-3), "unit": "recon/s", "ms_per_step": ms, "steps": steps,
           "precision": f"fp32 rows/FFT, cross-quadrant inverse {STENCIL_NAMES[stencil]}"}
    if ref is not None:
        got = x[0].cpu().numpy()
        out["rel_err_vs_fp64"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    del pipe
    return out


def extras(pkg, dev, args):
    """Short runs of the other workloads, appended to the batch line under their own keys (rank 0 of a one-GPU run):
    serve (p50/p99 latency and throughput at a rate the GPU sustains and at 2000 req/s), uneven (the 512-sinogram
    uneven batch in one CUDA graph) and large (N = 2048 at batch 1 and 8). Each reports its own accuracy against
    FP64 and its own clocks; none is part of the headline value."""
    import torch

    out = {}
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    invs, pool, setup = serve_setup(pkg, dev)
    runs = [serve_run(pkg, dev, invs, pool, rate, secs, seed=i)
            for i, (rate, secs) in enumerate(((150.0, 4.0), (2000.0, 1.0)))]
    out["serve"] = {"config": SERVE_CONFIG, "setup_s": setup, "sustained": runs[0], "at_2000_rps": runs[1],
                    "total_s": time.perf_counter() - t0}
    del invs, pool
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    out["uneven"] = dict(uneven_result(pkg, dev, 5, 3, tune_reps=1), config=UNEVEN_CONFIG,
                         total_s=time.perf_counter() - t0)
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    out["large"] = dict(large_result(pkg, dev, 3, 1), config=LARGE_CONFIG, total_s=time.perf_counter() - t0)
    return out


def _phantom_sinos(pkg, n, count, seed0, device, rel_sigma, ellipses=10, texture=0.0):
    """count seeded ellipse phantoms -> GPU ADRT (FP64) + i.i.d. noise rel_sigma[i] max|b_i|."""
    import torch

    N = 1 << n
    xs = np.stack([pkg.phantoms.ellipse_phantom(N, seed=seed0 + i, ellipses=ellipses, texture=texture)
                   for i in range(count)])
    b = pkg.adrtcore.adrt(n, torch.from_numpy(xs).to(device))
    g = torch.Generator(device=device).manual_seed(seed0)
    noise = torch.randn(b.shape, generator=g, device=device, dtype=b.dtype)
    sig = torch.as_tensor(np.broadcast_to(rel_sigma, (count,)).copy(), device=device).view(-1, 1, 1, 1)
    return b + sig * b.abs().amax(dim=(1, 2, 3), keepdim=True) * noise


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


SERVE_SIZES, SERVE_PROBS = [7, 8, 9, 10], [0.4, 0.3, 0.2, 0.1]
SERVE_SLOTS = {7: 64, 8: 64, 9: 32, 10: 16}


def serve_setup(pkg, dev):
    """The four hybrid inverses of the serving workload (N in {128, 256, 512, 1024}, p = 32, dense_cap 16) and a pool
    of 4 pinned noisy sinograms per size; returns (inverses, pool, setup seconds per N)."""
    setup, invs, pool = {}, {}, {}
    for n in SERVE_SIZES:
        t0 = time.perf_counter()
        invs[n] = pkg.FastHybridGpu(n, deg_cap=P_CAP, dense_cap=DENSE_CAP, precision="fp32", device=dev)
        setup[1 << n] = time.perf_counter() - t0
        pool[n] = [b.cpu().pin_memory() for b in _phantom_sinos(pkg, n, 4, 500 * n, dev, REL_SIGMA)]
    return invs, pool, setup


def serve_run(pkg, dev, invs, pool, rate, seconds, seed=0):
    """Continuous batching of Poisson(rate) hybrid-inverse requests for `seconds` (sizes drawn with SERVE_PROBS),
    120 GB HBM budget; p50/p99 latency (arrival to result on the host), throughput, and the first request of each
    size checked against the same sinogram inverted alone."""
    from adrt_pinv_gb300 import serve

    check = {}
    S = serve.InverseServer(lambda n: invs[n], lambda n: SERVE_SLOTS[n], hbm_budget_bytes=120e9, device=dev,
                            keep_result=lambda r: r.rid in check)
    for n in SERVE_SIZES:  # lanes (graph capture) and one warm batch each, before the clock starts
        S._admit_lane(n)
        for i in range(SERVE_SLOTS[n]):
            S.submit(serve.Request(-1, n, pool[n][i % 4]))
    while S.step():
        pass
    S.finished, S.max_busy = [], 0
    arr = serve.poisson_arrivals(rate, seconds, SERVE_SIZES, SERVE_PROBS, seed=seed)
    reqs, seen = [], set()
    for i, (t, n) in enumerate(arr):
        reqs.append((t, serve.Request(i, n, pool[n][i % 4])))
        if n not in seen:  # the first request of each size is checked against the same sinogram inverted alone
            seen.add(n)
            check[i] = reqs[-1][1]
    with ClockSampler(dev.index or 0) as clk:
        t0 = time.perf_counter()
        done = S.run(reqs)
        wall = time.perf_counter() - t0
    st = serve.InverseServer.stats(done)
    per = {}
    for n in SERVE_SIZES:
        d = [r for r in done if r.n == n]
        if d:
            per[1 << n] = serve.InverseServer.stats(d)
    same = max(_rel(r.result.numpy(), invs[r.n].apply(r.b.numpy())) for r in check.values())
    return {"offered_rps": len(arr) / seconds, "served_rps": st["throughput_rps"], "p50_ms": st["p50_ms"],
            "p99_ms": st["p99_ms"], "requests": st["requests"], "arrival_seconds": seconds, "wall_s": wall,
            "per_N": per, "max_concurrent_lanes": S.max_busy, "evictions": S.evictions,
            "lane_device_gb": S.memory_in_use() / 1e9, "served_vs_alone_rel_err": same, "clocks": clk.summary()}


SERVE_CONFIG = {"workload": "Poisson arrivals, N in {128,256,512,1024} w.p. {.4,.3,.2,.1}, hybrid, p=32, "
                            "dense_cap=16, FP32 rows + FP64 tables, 120 GB HBM budget",
                "slots": {str(1 << n): SERVE_SLOTS[n] for n in SERVE_SIZES}, "hbm_budget_gb": 120}


def run_serve(args):
    """The serving workload alone, at --serve-rate for --serve-seconds."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    dev = torch.device("cuda", 0)
    invs, pool, setup = serve_setup(pkg, dev)
    r = serve_run(pkg, dev, invs, pool, args.serve_rate, args.serve_seconds)
    line = {"metric": "served hybrid-inverse requests/s, mixed N (p50/p99 latency)", "value": r["served_rps"],
            "unit": "req/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded ellipse phantoms + Gaussian noise, 4 distinct sinograms per N)",
            "config": dict(SERVE_CONFIG, rate=args.serve_rate, seconds=args.serve_seconds), "setup_s": setup, **r}
    print(json.dumps(line), flush=True)


# dense rows per degree cap: without them the FP32 polynomial reaches 1e-5 at p = 16 (rows capped at 16 with high
# condition (Lambda + tau)/tau); at p = 8 the error stays near 3e-6 and dense rows would only add cost
UNEVEN_DENSE_CAP = {8: None, 16: 12, 32: DENSE_CAP, 64: DENSE_CAP}


def uneven_result(pkg, dev, steps, warmup, tune_reps=3):
    """512 sinograms, N uniform in {64, 128, 256, 512}, p in {8, 16, 32, 64}, method L_p / hybrid 50/50, noise
    sigma U[1e-4, 1e-2] max|b|, FP32 rows with FP64 tables: one CUDA graph over all 32 classes, every class's launch
    configuration autotuned first; accuracy of each class's first sinogram against the FP64 pipeline."""
    import torch

    from adrt_pinv_gb300 import inverse, tune, uneven
    rng = np.random.default_rng(2)
    total = 512
    ns = rng.choice([6, 7, 8, 9], size=total)
    ps = rng.choice([8, 16, 32, 64], size=total)
    ms = rng.choice(["lp", "hybrid"], size=total)
    sig = rng.uniform(1e-4, 1e-2, size=total)
    t0 = time.perf_counter()
    lam = {}
    invs, groups, sinos, keys = {}, [], [], []
    for n in (6, 7, 8, 9):
        for m in ("lp", "hybrid"):
            lam[(n, m)] = inverse.power_lam_max(n, 1 if m == "lp" else 2, 40, 1.5, dev)
            for p in (8, 16, 32, 64):
                idx = np.nonzero((ns == n) & (ps == p) & (ms == m))[0]
                if not len(idx):
                    continue
                cls = pkg.FastLpGpu if m == "lp" else pkg.FastHybridGpu
                inv = cls(n, lam_max=lam[(n, m)], deg_cap=p, dense_cap=UNEVEN_DENSE_CAP[p], precision="fp32",
                          device=dev)
                invs[(n, m, p)] = inv
                groups.append((inv, len(idx)))
                sinos.append(_phantom_sinos(pkg, n, len(idx), 10000 * n + 100 * p + (m == "lp"), dev, sig[idx]))
                keys.append((n, m, p))
    setup_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    U = uneven.UnevenBatch(groups, device=dev, tuner=tune.Tuner(reps=tune_reps), sinos=sinos)
    tune_s = time.perf_counter() - t1
    chosen = {}
    for key, tr in zip(keys, U.tuning):
        c = tr["config"]
        chosen[f"N={1 << key[0]} {key[1]} p={key[2]}"] = f"{c['dense']}/grid{c['row_grid']}"
    U.set_inputs(sinos)
    for _ in range(warmup):
        U.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index or 0) as clk:
        time.sleep(0.3)
        e0.record()
        for _ in range(steps):
            U.replay()
        e1.record()
        torch.cuda.synchronize()
    U.check()
    ms_step = e0.elapsed_time(e1) / steps
    # the same classes one after another, eager (no graph, no concurrency)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for pipe, x in zip(U.pipes, sinos):
        pipe.apply(x)
    torch.cuda.synchronize()
    eager_ms = (time.perf_counter() - t1) * 1e3
    outs = [o.clone() for o in U.replay()]
    # the same batch with every class's polynomial rows in one persistent launch per outer step (lock-step classes)
    t1 = time.perf_counter()
    P = uneven.PersistentUnevenBatch(groups, device=dev)
    P.set_inputs(sinos)
    for _ in range(warmup):
        P.replay()
    torch.cuda.synchronize()
    p_setup_s = time.perf_counter() - t1
    e0.record()
    for _ in range(steps):
        P.replay()
    e1.record()
    torch.cuda.synchronize()
    P.check()
    p_ms = e0.elapsed_time(e1) / steps
    p_outs = [o.clone() for o in P.replay()]
    errs, p_errs = {}, {}
    for key, inv, x, o, po in zip(keys, [g[0] for g in groups], sinos, outs, p_outs):
        ref = inv.pipeline(1, "fp64").apply(x[:1].contiguous())[0].cpu().numpy()
        errs[f"N={1 << key[0]} {key[1]} p={key[2]}"] = _rel(o[0].cpu().numpy(), ref)
        p_errs[f"N={1 << key[0]} {key[1]} p={key[2]}"] = _rel(po[0].cpu().numpy(), ref)
    del P
    return {"value": total / (ms_step * 1e-3), "unit": "recon/s", "steps": steps, "warmup": warmup,
            "ms_per_step": ms_step, "classes": len(groups), "eager_sequential_ms": eager_ms,
            "graph_launches_per_step": 1, "setup_s": setup_s, "autotune_s": tune_s, "autotuned": chosen,
            "device_gb": U.device_bytes() / 1e9, "max_rel_err_vs_fp64": max(errs.values()), "rel_err_vs_fp64": errs,
            "persistent_rows": {"value": total / (p_ms * 1e-3), "unit": "recon/s", "ms_per_step": p_ms,
                                "setup_s": p_setup_s, "max_rel_err_vs_fp64": max(p_errs.values()),
                                "how": "classes in lock-step, one persistent row launch per outer step for all of "
                                       "them, one CUDA graph; launch configurations not autotuned"},
            "clocks": clk.summary()}


UNEVEN_CONFIG = {"workload": "512 sinograms, N U{64,128,256,512}, p U{8,16,32,64}, L_p/hybrid 50/50, "
                             "dense_cap 16 (12 at p=16, none at p=8), FP32 rows + FP64 tables, one CUDA graph"}


def run_uneven(args):
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    r = uneven_result(pkg, torch.device("cuda", 0), args.steps, args.warmup)
    line = {"metric": "uneven-batch inverse recon/s (one CUDA graph, 32 N/p/method classes)", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded ellipse phantoms + Gaussian noise sigma U[1e-4,1e-2] max|b|)",
            "config": UNEVEN_CONFIG, **r}
    print(json.dumps(line), flush=True)


def large_result(pkg, dev, steps, warmup, profile_region=False, high_rows="dense"):
    """N = 2048 (n = 11), hybrid, p = 64, dense_cap 16, FP32 rows with FP64 tables, batch 1 and 8; 40 ellipses plus
    a 0.1-weighted uniform texture; relative error of the first image against the FP64 pipeline on the same plan.
    high_rows: the rows with d_k > 16 as dense operators ("dense") or as compensated float-float rows ("ff")."""
    import torch

    n = 11
    t0 = time.perf_counter()
    H = pkg.FastHybridGpu(n, deg_cap=64, dense_cap=DENSE_CAP, precision="fp32", device=dev, high_rows=high_rows)
    setup_s = time.perf_counter() - t0
    b = _phantom_sinos(pkg, n, 8, 777, dev, REL_SIGMA, ellipses=40, texture=0.1)
    res = {}
    with ClockSampler(dev.index or 0) as clk:
        for B in (1, 8):
            pipe = H.pipeline(B).capture()
            x = b[:B].contiguous()
            for _ in range(max(1, warmup)):
                pipe.replay(x)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            k = max(1, min(steps, 5))
            e0.record()
            for _ in range(k):
                pipe.replay(x)
            e1.record()
            torch.cuda.synchronize()
            ms_b = e0.elapsed_time(e1) / k
            res[f"batch{B}"] = {"ms_per_apply": ms_b, "recon_s": B / (ms_b * 1e-3)}
    if profile_region:  # one more batch-8 replay as the profiled region (per-kernel launch lists)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        pipe.replay(b[:8].contiguous())
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    got = pipe.x_out[0].cpu().numpy()
    ref = H.pipeline(1, "fp64").apply(b[:1].contiguous())[0].cpu().numpy()
    H.pipeline(8).tables.raise_if_error()
    return {"results": res, "setup_s": setup_s, "outer_deg": H.outer_deg, "n_dense_freqs": H.eng.n_dense,
            "high_rows": high_rows, "device_gb": H.pipeline(8).device_bytes() / 1e9,
            "rel_err_vs_fp64": _rel(got, ref), "clocks": clk.summary()}


LARGE_CONFIG = {"workload": "hybrid inverse N=2048, p=64, dense_cap=16, batch 1 and 8, FP32 rows + FP64 tables, "
                            "40 seeded ellipses + 0.1 uniform texture, noise 1e-3 max|b|"}


def run_large(args):
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    r = large_result(pkg, torch.device("cuda", 0), args.steps, args.warmup, args.profile_region, args.high_rows)
    line = {"metric": "hybrid-inverse recon/s at N=2048 (batch 8)", "value": r["results"]["batch8"]["recon_s"],
            "unit": "recon/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": LARGE_CONFIG, **r}
    print(json.dumps(line), flush=True)


def run_adrt(args):
    """The spatial ADRT (int32, forward and transpose) and CGLS iterations alone: their HBM rates."""
    import torch

    import __graft_entry__ as ge

    pkg = ge.load_package()
    line = {"metric": "spatial ADRT int32 images/s and CGLS image-iterations/s at N=256", "n_gpus": 1,
            "adrt_int32": adrt_int32_timing(pkg, args.n, args.batch, args.steps, torch),
            "cgls": cgls_timing(pkg, args.n, 16, 50, torch)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.mode == "serve":
        run_serve(a)
    elif a.mode == "uneven":
        run_uneven(a)
    elif a.mode == "large":
        run_large(a)
    elif a.mode == "adrt":
        run_adrt(a)
    else:
        run_ours(a)
