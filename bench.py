"""Benchmark of the batched LCA module on one GB300 (and N replicas under torchrun).

Workload (the headline metric's configuration): 256 images of 32x32x3 with a seeded 1/f
amplitude spectrum and random phase, each normalised to zero mean and unit std; an LCA
layer of 16x16x512 (stride 2) with a dictionary of 512 features of 8x8x3, N(0,1) then
L2-normalised; VThresh = AShift = 0.15, AMin = 0, tau = 100, dt = 1; 400 timesteps per
solve, the last 50 with BF16x3 split products.  One bench step = one full solve of the
batch (reset, 400 timesteps, the FP64 probe energy).  Synthetic data stands in for
natural images; inputs are generated here from fixed seeds.

Metric: images*timesteps per second of the BF16 tensor-core form (value, device-resident
inputs), the same through the C ABI with host buffers (e2e), the plain FP32 form beside it,
the final-energy error against the FP64 oracle, the dominant kernel's roofline fraction
(CUDA events around every launch in the timed region), the presynaptic sparse-delivery
microbenchmark, and the CPU oracle timed on this host's cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(nbatch=256, in_shape=(32, 32, 3), v1_shape=(16, 16, 512), nxp=8, VThresh=0.15, AMin=0.0, AShift=0.15,
           VWidth=0.0, tau=100.0, dt=1.0, timesteps=400, x3_steps=50, seed=1237)
METRIC = "LCA images*steps/s BF16-TC vs plain FP32 at <=1e-3 energy err; delivery HBM GB/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return dict(PEAKS_FALLBACK, source="fallback")


# ---------------------------------------------------------------------------------------------
# synthetic inputs
# ---------------------------------------------------------------------------------------------
def one_over_f_images(rng, nb, ny, nx, c):
    fy = np.fft.fftfreq(ny)[:, None]
    fx = np.fft.fftfreq(nx)[None, :]
    f = np.sqrt(fy ** 2 + fx ** 2)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    ph = rng.uniform(0, 2 * np.pi, (nb, c, ny, nx))
    img = np.real(np.fft.ifft2(amp[None, None] * np.exp(1j * ph)))  # [nb][c][ny][nx]
    img = np.transpose(img, (0, 2, 3, 1))
    mu = img.mean(axis=(1, 2, 3), keepdims=True)
    sd = img.std(axis=(1, 2, 3), keepdims=True)
    return np.ascontiguousarray(((img - mu) / sd).astype(np.float32))


def dictionary(rng, nf, p, c):
    w = rng.normal(size=(nf, p, p, c))
    w /= np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))
    return w.astype(np.float32)


def make_inputs(cfg, nb=None, seed_offset=0):
    """The dictionary (one model, the same on every rank) and an image shard (seed + 1 + offset)."""
    nb = cfg["nbatch"] if nb is None else nb
    w = dictionary(np.random.default_rng(cfg["seed"]), cfg["v1_shape"][2], cfg["nxp"], cfg["in_shape"][2])
    x = one_over_f_images(np.random.default_rng(cfg["seed"] + 1 + seed_offset), nb, *cfg["in_shape"])
    return w, x


# ---------------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [t.strip() for t in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# CPU oracle timing (the reference's CPU path restated; test infrastructure)
# ---------------------------------------------------------------------------------------------
def oracle_lca_params(O, cfg, nb):
    (iy, ix, ic), (vy, vx, vf) = cfg["in_shape"], cfg["v1_shape"]
    return O.lca_params(nbatch=nb, inNx=ix, inNy=iy, inNf=ic, v1Nx=vx, v1Ny=vy, v1Nf=vf, nxp=cfg["nxp"],
                        nyp=cfg["nxp"], VThresh=cfg["VThresh"], AShift=cfg["AShift"], AMin=cfg["AMin"],
                        VWidth=cfg["VWidth"], tau=cfg["tau"], dtFixed=cfg["dt"])


def cpu_sample(cfg, threads, warm_steps, timed_steps):
    """The oracle (FP32, reference order) on `threads` images, one per thread: warm_steps untimed
    timesteps into the dynamics, then timed_steps timed.  Returns images*steps/s."""
    from oracle import oracle as O
    O.build()
    w, x = make_inputs(cfg, nb=threads, seed_offset=100)
    p = oracle_lca_params(O, cfg, threads)
    v = np.zeros((threads,) + cfg["v1_shape"], np.float32)
    if warm_steps:
        v, _, _, _ = O.lca_run(p, w, x[None], warm_steps, v, threads=threads, want_recon=False)
    t0 = time.perf_counter()
    O.lca_run(p, w, x[None], timed_steps, v, threads=threads, want_recon=False)
    dt = time.perf_counter() - t0
    return threads * timed_steps / dt, dt


def fp64_energy(cfg, x, w, nimg, threads):
    from oracle import oracle as O
    O.build()
    p = oracle_lca_params(O, cfg, nimg)
    v0 = np.zeros((nimg,) + cfg["v1_shape"])
    _, _, _, e = O.lca_run(p, w.astype(np.float64), x[None, :nimg].astype(np.float64), cfg["timesteps"], v0,
                           f64=True, threads=threads, want_recon=False)
    return e[-1]


# ---------------------------------------------------------------------------------------------
# replicas over the batch: each rank solves its own shard; only timings cross ranks
# ---------------------------------------------------------------------------------------------
def shard_seed_offset(rank):
    """Rank r solves its own 256-image shard, generated from seed + r."""
    return rank


def max_over_ranks(ms, dist, device):
    """Slowest rank's time (the job finishes when the last replica does)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, nb, timesteps, ms):
    """Whole-job images*timesteps per second: all ranks' images over the slowest rank's time."""
    return world * nb * timesteps / (ms / 1000.0)


# ---------------------------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    cfg = CFG
    from oracle import oracle as O
    O.build()
    w, x = make_inputs(cfg, nb=cores, seed_offset=100)
    p = oracle_lca_params(O, cfg, cores)
    v = np.zeros((cores,) + cfg["v1_shape"], np.float32)
    per_step = 25  # timesteps per bench step; the dynamics continue from step to step
    for _ in range(args.warmup):
        v, _, _, _ = O.lca_run(p, w, x[None], per_step, v, threads=cores, want_recon=False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, _, _, _ = O.lca_run(p, w, x[None], per_step, v, threads=cores, want_recon=False)
    dt = time.perf_counter() - t0
    value = cores * per_step * args.steps / dt
    sample = (f"{cores} images x {per_step} timesteps per step (one image per thread), continuing the dynamics "
              f"after {args.warmup * per_step} warm-up timesteps; same layer sizes as the GPU workload")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "images*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched LCA 256x32x32x3 -> 16x16x512, 8x8x3 dictionary, 400 timesteps",
                       "reference_sample": sample},
            "cpu_baseline": {"value": value, "unit": "images*steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "images*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# plain LCA, batch 1 (32x32x1 -> 16x16x64, 8x8x1 features, 200 timesteps): absolute latency
# ---------------------------------------------------------------------------------------------
def config1_bench(torch, capi, steps=200, reps=5):
    """Latency of one timestep of the plain LCA configuration at batch 1, four ways: the C ABI
    entry points composed in the reference's phase order (what the reference's GPU layer and
    delivery classes call per timestep: error accumulate + identity threshold, postsynaptic
    delivery, LCA update + threshold, compaction, presynaptic sparse delivery, energy probes),
    launched one by one and as one captured CUDA graph of the 200 timesteps; the LCA solver's
    FP32 and BF16 forms; and the CPU oracle on one core."""
    import time
    from oracle import oracle as O
    rng = np.random.default_rng(1234 + 1)
    x_np = rng.uniform(0.0, 1.0, (1, 32, 32, 1))
    x_np = (x_np - x_np.mean()).astype(np.float32)
    w_np = rng.normal(size=(64, 8, 8, 1))
    w_np = (w_np / np.sqrt((w_np ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)
    vt, inf = 0.1, float("inf")
    v1 = capi.Loc.make(1, 16, 16, 64, 2)
    er = capi.Loc.make(1, 32, 32, 1, 3)
    wd = torch.from_numpy(w_np).cuda()
    xd = torch.from_numpy(x_np).cuda()
    pre_conn, post_conn = capi.conn_desc(v1, er, 8, 8), capi.conn_desc(er, v1, 4, 4)
    v = torch.zeros(v1.res_shape(), device="cuda")
    a1 = torch.zeros(v1.ext_shape(), device="cuda")
    gsyn_e = torch.zeros((2,) + er.res_shape(), device="cuda")
    ge = torch.zeros(er.res_shape(), device="cuda")
    ae = torch.zeros(er.ext_shape(), device="cuda")
    g1 = torch.zeros(v1.res_shape(), device="cuda")
    ent = torch.zeros((1, v1.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(1, dtype=torch.int64, device="cuda")
    scr = torch.empty(capi.lib().pvgpu_compact_scratch_bytes(1, v1.num_ext), dtype=torch.uint8, device="cuda")
    dt = torch.ones(1, dtype=torch.float64, device="cuda")
    l2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    l1 = torch.zeros(1, dtype=torch.float64, device="cuda")

    def reset():
        v.zero_()
        capi.ann_activity(v1, v, vt, 0.0, inf, vt, 0.0, a1)
        gsyn_e.zero_()
        gsyn_e[0].copy_(xd)

    def timestep(mode):
        capi.gsyn_accumulate(er.num_res, [1.0, -1.0], gsyn_e, ge)
        capi.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0, ae)
        g1.zero_()
        capi.deliver_post(post_conn, ae, wd, g1, mode=mode)
        capi.lca_update(v1, True, dt, 100.0, g1, a1, v)
        capi.ann_activity(v1, v, vt, 0.0, inf, vt, 0.0, a1)
        capi.compact_active(a1, 1, v1.num_ext, ent, num, scratch=scr)
        gsyn_e[1].zero_()
        capi.deliver_pre(pre_conn, wd, gsyn_e[1], entries=ent, num_active=num, mode=mode)
        capi.cost_sum(er, ae, capi.COST_L2, 0.0, 0.0, l2)
        capi.cost_sum(v1, a1, capi.COST_L1, 0.0, 0.0, l1)

    def events_ms(fn, n=reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    out = {"workload": "plain LCA, batch 1: 32x32x1 uniform[0,1] minus its mean -> V1 16x16x64 stride 2, 64 x 8x8x1 "
                       "N(0,1) L2-normalised, VThresh=AShift=0.1, AMin=0, tau=100, dt=1, 200 timesteps",
           "timesteps": steps}
    per_mode = {}
    for name, mode in (("reference_order", capi.DELIVER_REFERENCE_ORDER), ("fast", capi.DELIVER_FAST)):
        def run_all(mode=mode):
            reset()
            for _ in range(steps):
                timestep(mode)
        launched_ms = events_ms(run_all, 2)
        reset()
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr):
            for _ in range(steps):
                timestep(mode)
        graph_ms = events_ms(lambda: (reset(), gr.replay()))
        per_mode[name] = {"launched_ms_per_step": launched_ms / steps, "graph_ms_per_step": graph_ms / steps,
                          "kernels_per_step": 11}
        del gr
    out["c_abi_composed"] = per_mode
    for name, prec, x3 in (("fp32_solver", capi.LCA_FP32, 0), ("bf16_solver", capi.LCA_BF16, 25)):
        s = capi.LcaSolver(1, (32, 32, 1), (16, 16, 64), 8, vt)
        s.set_weights(wd)

        def solve(s=s, prec=prec, x3=x3):
            s.reset()
            s.run(xd, steps, x3_steps=x3, precision=prec)
        ms = events_ms(solve)
        assert s.error_flag() == 0
        out[name] = {"ms_per_step": ms / steps, "image_steps_per_s": steps / (ms / 1e3)}
        if x3:
            out[name]["bf16x3_last_steps"] = x3
        s.close()
    p = O.lca_params()
    t0 = time.perf_counter()
    O.lca_run(p, w_np, x_np[None], steps, np.zeros((1, 16, 16, 64), np.float32), want_recon=False)
    cpu_s = time.perf_counter() - t0
    out["cpu_oracle"] = {"ms_per_step": cpu_s * 1e3 / steps, "cores": 1, "kind": "port",
                         "sample": "oracle, the whole 200-timestep run at batch 1 on one core"}
    return out


# ---------------------------------------------------------------------------------------------
# delivery microbenchmark (presynaptic sparse delivery, 128x128x256 -> 128x128x64, 7x7, batch 16)
# ---------------------------------------------------------------------------------------------
def delivery_bench(torch, capi, reps=5):
    """Presynaptic delivery of the 16 x (128x128x256 -> 128x128x64), 7x7 workload at three
    densities: the sparse kernel from the SparseList, the tensor-core kernel from the dense
    activity (split-TF32, density-independent), and the faster of the two; then the
    postsynaptic delivery of the same connection, FP32 SIMT and tensor-core."""
    nb = 16
    pre = capi.Loc.make(nb, 128, 128, 256, 3)
    post = capi.Loc.make(nb, 128, 128, 64, 0)
    conn = capi.conn_desc(pre, post, 7, 7)
    g = torch.Generator(device="cuda").manual_seed(1234 + 2)
    w = (torch.randn(256 * 7 * 7 * 64, device="cuda", generator=g) * 0.05).contiguous()
    gsyn = torch.zeros(post.res_shape(), device="cuda")
    gtc = torch.zeros(post.res_shape(), device="cuda")
    entries = torch.empty((nb, pre.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(nb, dtype=torch.int64, device="cuda")
    ws = torch.empty(capi.deliver_tc_workspace_bytes(conn), dtype=torch.uint8, device="cuda")

    def timed(fn, n):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    def graph_timed(fn, n, reps=3):
        # n calls captured in one CUDA graph, so that host launch overhead does not show in
        # the time of a kernel that runs for tens of microseconds
        fn()
        torch.cuda.synchronize()
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr):
            for _ in range(n):
                fn()
        gr.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            gr.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / (reps * n)

    hbm_peak = peaks()["hbm_gbs"]
    cscratch = torch.empty(capi.lib().pvgpu_compact_scratch_bytes(nb, pre.num_ext), dtype=torch.uint8,
                           device="cuda")
    dense_flops = 2 * nb * 128 * 128 * 64 * 49 * 256
    out = {}
    for p in (0.01, 0.05, 0.2):
        a = torch.zeros(pre.ext_shape(), device="cuda")
        core = (torch.rand((nb, 128, 128, 256), device="cuda", generator=g) < p).float() * \
            (1.0 - torch.rand((nb, 128, 128, 256), device="cuda", generator=g))
        a[:, 3:131, 3:131, :] = core
        capi.compact_active(a, nb, pre.num_ext, entries, num)
        torch.cuda.synchronize()
        nnz = int(num.sum().item())
        ms = timed(lambda: capi.deliver_pre(conn, w, gsyn, entries=entries, num_active=num), reps)
        # algorithmic bytes: entries read, GSyn read+write, weights once
        byts = 8 * nnz + 8 * post.num_res * nb + 4 * w.numel()
        flops = 2 * nnz * 7 * 7 * 64
        cms = graph_timed(lambda: capi.compact_active(a, nb, pre.num_ext, entries, num, scratch=cscratch), 10)
        cbytes = 4 * pre.num_ext * nb + 8 * nnz  # one read of the activity + entries written
        tms = timed(lambda: capi.deliver_pre_tc(conn, a, w, gtc, ws), reps)
        # size-independent check at full size: both kernels from zero give the same GSyn
        gsyn.zero_()
        gtc.zero_()
        capi.deliver_pre(conn, w, gsyn, entries=entries, num_active=num)
        capi.deliver_pre_tc(conn, a, w, gtc, ws)
        torch.cuda.synchronize()
        rel = float((gsyn - gtc).abs().max().item() / max(gsyn.abs().max().item(), 1e-30))
        out[str(p)] = {"nnz_per_image": nnz / nb, "ms": ms, "GB_s": byts / ms / 1e6, "GFLOP_s": flops / ms / 1e6,
                       "compaction_ms": cms, "compaction_GB_s": cbytes / cms / 1e6,
                       "compaction_frac_of_measured_hbm": cbytes / cms / 1e6 / hbm_peak,
                       "tc_ms": tms, "tc_dense_TFLOP_s": dense_flops / tms / 1e9,
                       "best_ms": min(ms, tms), "best": "sparse" if ms <= tms else "tensor-core",
                       "sparse_vs_tc_max_rel_diff": rel}
    capi.deliver_tc_check_error()
    out["cpu_baseline"] = delivery_cpu_baseline(w)
    # postsynaptic perspective, dense activity (p = 0.2 from above), post weights on the device
    wpost = torch.zeros_like(w)
    capi.transpose_weights(conn, w, wpost)
    fp32_ms = timed(lambda: capi.deliver_post(conn, a, wpost, gsyn), 1)
    tc_ms = timed(lambda: capi.deliver_post_tc(conn, a, wpost, gtc, ws), reps)
    out["post"] = {"fp32_ms": fp32_ms, "tc_ms": tc_ms, "fp32_TFLOP_s": dense_flops / fp32_ms / 1e9,
                   "tc_TFLOP_s": dense_flops / tc_ms / 1e9, "speedup_tc_over_fp32": fp32_ms / tc_ms,
                   "tc_tf32_products_per_term": 3}
    return out


def delivery_cpu_baseline(w):
    """The reference's CPU deliveries for the delivery workload, as the oracle's ports of
    PresynapticPerspectiveConvolveDelivery (SparseList branch) and
    PostsynapticPerspectiveConvolveDelivery (each pinned bit for bit to the reference's own code
    compiled from its tree): one image per thread, on one core and on all host cores.  Bounded
    samples: the presynaptic delivery of one full image at p = 0.01 (the timed density) per
    thread; the postsynaptic delivery of a 32x32 crop of the same connection per thread, scaled
    to a 128x128 image by the output count (its cost per output does not depend on the size)."""
    import concurrent.futures as cf
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    wn = w.detach().cpu().numpy().reshape(256, 7, 7, 64)
    pre1 = O.Loc.make(1, 128, 128, 256, 3)
    post1 = O.Loc.make(1, 128, 128, 64, 0)
    rng = np.random.default_rng(1234 + 2)
    core = (rng.random((128, 128, 256)) < 0.01) * (1.0 - rng.random((128, 128, 256)))
    a1 = np.zeros(pre1.ext_shape(), np.float32)
    a1[0, 3:131, 3:131, :] = core
    ent, num = O.compact(a1)

    def pre_one(_):
        t0 = time.perf_counter()
        O.deliver_pre(pre1, post1, 7, 7, wn, entries=ent, num_active=num)
        return time.perf_counter() - t0

    # 32x32 crop for the postsynaptic loop (dense activity, p = 0.2 as in the GPU figure)
    preC = O.Loc.make(1, 32, 32, 256, 3)
    postC = O.Loc.make(1, 32, 32, 64, 0)
    aC = np.zeros(preC.ext_shape(), np.float32)
    aC[0, 3:35, 3:35, :] = (rng.random((32, 32, 256)) < 0.2) * (1.0 - rng.random((32, 32, 256)))
    w_post = O.transpose_shared(preC, postC, 7, 7, wn)

    def post_one(_):
        t0 = time.perf_counter()
        O.deliver_post(preC, postC, 7, 7, w_post, aC)
        return time.perf_counter() - t0

    out = {}
    for name, fn, scale in (("pre_sparse_p0.01", pre_one, 1.0), ("post_dense", post_one, 16.0)):
        t1 = fn(0)  # one core, one image (post: 16 crops = one 128x128 image)
        with cf.ThreadPoolExecutor(cores) as ex:
            t0 = time.perf_counter()
            list(ex.map(fn, range(cores)))
            tall = time.perf_counter() - t0
        ms_batch_1 = 16 * scale * t1 * 1e3               # 16 images on one core
        ms_batch_all = 16 * scale * tall / cores * 1e3   # 16 images spread over all cores
        out[name] = {"ms_per_16_image_batch_1_core": ms_batch_1,
                     "ms_per_16_image_batch_all_cores": ms_batch_all, "cores": cores, "kind": "port",
                     "sample": ("one 128x128x256 image at p = 0.01 per thread" if scale == 1.0 else
                                "a 32x32 crop per thread, scaled by 16 to a 128x128 image")}
    return out


# ---------------------------------------------------------------------------------------------
# LIF spiking network (the spiking configuration): 8 images, 1000 timesteps in one CUDA graph
# ---------------------------------------------------------------------------------------------
def gaussian_weights(torch, nfpre, p, nfpost, sigma, peak, device="cuda"):
    r = torch.arange(p, device=device, dtype=torch.float32) - (p - 1) / 2.0
    g = torch.exp(-(r[:, None] ** 2 + r[None, :] ** 2) / (2 * sigma ** 2))
    return (peak * g[None, :, :, None].expand(nfpre, p, p, nfpost)).contiguous()


class LifNet:
    """Input (256x256x1 Poisson spikes, rates U[5, 50] Hz at dt = 1 ms, pre-generated on the device
    as dense frames and compacted each step) -> excitatory LIF 256x256x32 (11x11 Gaussian, sigma 3,
    peak 0.5, EXC channel) -> inhibitory LIF 128x128x8 (stride 2, 3x3 weights 0.05, EXC channel)
    -> back to the excitatory layer (8x8 Gaussian, sigma 2, peak 1.0, INH channel; one-to-many at
    stride 2 needs an even patch, so 8 rather than 7).  Default LIF parameters, arma method, noise
    off.  One step: compact the input frame, the three deliveries (presynaptic, from SparseLists),
    the two LIF updates, the compaction of each layer's spikes."""

    def __init__(self, torch, capi, nb=8, steps=1000, seed=1234 + 5):
        self.t, self.c, self.nb, self.steps = torch, capi, nb, steps
        n, ne, ni = 256, 32, 8
        self.inp = capi.Loc.make(nb, n, n, 1, 5)
        self.exc = capi.Loc.make(nb, n, n, ne, 2)
        self.inh = capi.Loc.make(nb, n // 2, n // 2, ni, 2)
        exc_res = capi.Loc.make(nb, n, n, ne, 0)
        inh_res = capi.Loc.make(nb, n // 2, n // 2, ni, 0)
        self.c_in_exc = capi.conn_desc(self.inp, exc_res, 11, 11)
        self.c_exc_inh = capi.conn_desc(self.exc, inh_res, 3, 3)
        self.c_inh_exc = capi.conn_desc(self.inh, exc_res, 8, 8)
        self.w_in_exc = gaussian_weights(torch, 1, 11, ne, 3.0, 0.5)
        self.w_exc_inh = torch.full((ne * 4, 3, 3, ni), 0.05, device="cuda")  # 4 kernel phases x 32 features
        self.w_inh_exc = gaussian_weights(torch, ni, 8, ne, 2.0, 1.0)
        g = torch.Generator(device="cuda").manual_seed(seed)
        rates = 5.0 + 45.0 * torch.rand((nb, n, n, 1), device="cuda", generator=g)
        self.frames = torch.zeros((steps,) + tuple(self.inp.ext_shape()), device="cuda")
        self.frames[:, :, 5:5 + n, 5:5 + n, :] = (torch.rand((steps, nb, n, n, 1), device="cuda", generator=g)
                                                  < rates * 1e-3).float()
        self.layers = {}
        for name, loc in (("in", self.inp), ("exc", self.exc), ("inh", self.inh)):
            d = {"loc": loc,
                 "ent": torch.zeros((nb, loc.num_ext, 2), dtype=torch.int32, device="cuda"),
                 "num": torch.zeros(nb, dtype=torch.int64, device="cuda"),
                 "scratch": torch.empty(max(1, capi.lib().pvgpu_compact_scratch_bytes(nb, loc.num_ext)),
                                        dtype=torch.uint8, device="cuda")}
            if name != "in":
                nres = nb * loc.nx * loc.ny * loc.nf
                d.update(rnd=torch.zeros((nres, 4), dtype=torch.int32, device="cuda"),
                         V=torch.full((nres,), -70.0, device="cuda"), Vth=torch.full((nres,), -55.0, device="cuda"),
                         GE=torch.zeros(nres, device="cuda"), GI=torch.zeros(nres, device="cuda"),
                         GIB=torch.zeros(nres, device="cuda"), gs=torch.zeros((3, nres), device="cuda"),
                         A=torch.zeros(loc.ext_shape(), device="cuda"), spikes=torch.zeros(nres, device="cuda"))
                capi.taus_init(d["rnd"], nres, 17 if name == "exc" else 18)
            self.layers[name] = d
        self.prm = capi.LifParams.make()

    def compact(self, d, a):
        self.c.compact_active(a, self.nb, d["loc"].num_ext, d["ent"], d["num"], scratch=d["scratch"])

    def step(self, i, ev=None):
        c, L = self.c, self.layers
        rec = (lambda k: ev[k].record()) if ev else (lambda k: None)
        rec(0)
        self.compact(L["in"], self.frames[i])
        e, h = L["exc"], L["inh"]
        e["gs"].zero_()
        h["gs"].zero_()
        c.deliver_pre(self.c_in_exc, self.w_in_exc, e["gs"][0], entries=L["in"]["ent"], num_active=L["in"]["num"])
        c.deliver_pre(self.c_inh_exc, self.w_inh_exc, e["gs"][1], entries=h["ent"], num_active=h["num"])
        rec(1)
        c.lif_update(e["loc"], "a", self.prm, 1.0, e["rnd"], e["V"], e["Vth"], e["GE"], e["GI"], e["GIB"], e["gs"], e["A"])
        rec(2)
        self.compact(e, e["A"])
        c.deliver_pre(self.c_exc_inh, self.w_exc_inh, h["gs"][0], entries=e["ent"], num_active=e["num"])
        c.lif_update(h["loc"], "a", self.prm, 1.0, h["rnd"], h["V"], h["Vth"], h["GE"], h["GI"], h["GIB"], h["gs"], h["A"])
        self.compact(h, h["A"])
        rec(3)


def dictlearn_bench(torch, capi, reps=5):
    """Differentiable dictionary learning at full size: 32 images 64x64x1 (1/f, unit std), V1
    16x16x256 stride 4, 256 features of 16x16x1, 100 unrolled LCA timesteps from V = 0 with a
    checkpoint every 10, loss 0.5 ||x - W^T a||^2 + 0.1 ||a||_1; one gradient = the forward pass,
    the recomputation of each checkpointed segment and the adjoint pass, through the C ABI
    (pvgpu_lca_grad_run: one CUDA graph).  CPU baseline: the reference's own learning step on the
    host cores -- the LCA solve of the oracle (one image per thread) for a sample of the batch --
    since the reference learns dictionaries with the Hebbian rule after an LCA solve."""
    import time
    from oracle import oracle as O
    rng = np.random.default_rng(1234 + 4)
    nb, n, v1, P, T, lam = 32, 64, (16, 16, 256), 16, 100, 0.1
    w = rng.normal(size=(v1[2], P, P, 1))
    w = (w / np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)
    f = np.sqrt(np.fft.fftfreq(n)[:, None] ** 2 + np.fft.fftfreq(n)[None, :] ** 2)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    xi = np.real(np.fft.ifft2(amp[None] * np.exp(1j * rng.uniform(0, 2 * np.pi, (nb, n, n)))))
    xi = (xi - xi.mean(axis=(1, 2), keepdims=True)) / xi.std(axis=(1, 2), keepdims=True)
    x_np = np.ascontiguousarray(xi[..., None].astype(np.float32))
    x = torch.from_numpy(x_np).cuda()
    wd = torch.from_numpy(w).cuda()
    dw = torch.empty_like(wd)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = capi.LcaGrad(nb, (n, n, 1), v1, P, lam, lam, T, checkpoint_every=10)
    grad.run(wd, x, dw, loss)  # captures the graph
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        grad.run(wd, x, dw, loss)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    M, F, KP = nb * v1[0] * v1[1], v1[2], P * P
    flops = (8 * T + 3) * 2 * M * F * KP  # every GEMM of the forward, the recomputation and the adjoint
    # CPU: the oracle's LCA solve of the same geometry, one image per thread, on a sample
    cores = min(os.cpu_count() or 1, nb)
    p = O.lca_params(nbatch=cores, inNx=n, inNy=n, inNf=1, v1Nx=v1[1], v1Ny=v1[0], v1Nf=v1[2], nxp=P, nyp=P,
                     VThresh=lam, AShift=lam, AMin=0.0, tau=100.0)
    cpu_steps = 5
    t0 = time.perf_counter()
    O.lca_run(p, w, x_np[None, :cores], cpu_steps, np.zeros((cores,) + v1, np.float32), threads=cores,
              want_recon=False)
    cpu_s = time.perf_counter() - t0
    emulated = bool(grad.emulated_fp32())
    fp32_tf = flops / (ms / 1000.0) / 1e12
    # the emulated FP32 GEMM issues 9 BF16 products per FP32 product (each operand in three BF16
    # parts); averaged over the whole gradient (the fold / im2col / update kernels included)
    issued = fp32_tf * (9 if emulated else 1)
    pk = peaks()
    roofline = ({"bound": "tensor", "achieved": issued, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                 "frac": issued / pk["bf16_tflops"], "peak_source": pk.get("source", "fallback"),
                 "what": "BF16 products issued by the GEMMs, averaged over the whole gradient"}
                if emulated else None)
    return {"workload": "32 x 64x64x1 -> V1 16x16x256 stride 4, 256 x 16x16x1 dictionary, 100 unrolled "
                        "timesteps (checkpoint every 10), gradient of 0.5||x - W^T a||^2 + 0.1||a||_1 w.r.t. W",
            "ms_per_gradient": ms, "image_steps_per_s": nb * T / (ms / 1000.0), "loss": float(loss.item()),
            "grad_norm": float(dw.norm().item()), "dtype": "f32",
            "gemm_math": "fp32 emulated on bf16 tensor cores" if emulated else "fp32",
            "gemm_tflops_fp32_equivalent": fp32_tf, "roofline": roofline,
            "cpu_baseline": {"value": cores * cpu_steps / cpu_s, "unit": "image-steps/s", "cores": cores,
                             "kind": "port", "sample": f"oracle LCA solve (forward only) of {cores} images x "
                                                       f"{cpu_steps} timesteps, one image per thread "
                                                       f"({cpu_s:.1f} s)"}}


def lif_bench(torch, capi, steps=1000, cpu_sample=True):
    nb = 8
    net = LifNet(torch, capi, nb=nb, steps=steps)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for i in range(3):  # warm-up, uncaptured
            net.step(i)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for i in range(steps):
            net.step(i)
    torch.cuda.synchronize()
    graph.replay()  # warm-up replay
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    graph.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # per-phase split of one step (outside the graph)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    k, t_in, t_lif, t_rest = 10, 0.0, 0.0, 0.0
    for i in range(k):
        net.step(i, ev)
        torch.cuda.synchronize()
        t_in += ev[0].elapsed_time(ev[1])
        t_lif += ev[1].elapsed_time(ev[2])
        t_rest += ev[2].elapsed_time(ev[3])
    ex, ih = net.layers["exc"], net.layers["inh"]
    exc_n = nb * 256 * 256 * 32
    out = {"workload": "8 images: Poisson input 256x256x1 (U[5,50] Hz, dt 1 ms) -> exc LIF 256x256x32 (11x11 Gaussian "
                       "sigma 3 peak 0.5) -> inh LIF 128x128x8 (stride 2, 3x3) -> exc (INH channel, 8x8 Gaussian sigma 2 "
                       "peak 1); arma, noise off; 1000 timesteps in one CUDA graph",
           "timesteps": steps, "graph_ms": ms, "ms_per_step": ms / steps, "image_steps_per_s": nb * steps / (ms / 1e3),
           "exc_spikes_per_image_step": float(ex["num"].float().mean().item()),
           "inh_spikes_per_image_step": float(ih["num"].float().mean().item()),
           "split_ms": {"input_compaction_and_exc_deliveries": t_in / k, "exc_lif_update": t_lif / k,
                        "exc_compaction_inh_delivery_update_compaction": t_rest / k},
           "exc_lif_update_GB_s": exc_n * 88 / (t_lif / k) / 1e6}
    if cpu_sample:
        out["cpu_oracle"] = lif_cpu_sample()
        t = max(1, min(nb, os.cpu_count() or 1))
        out["cpu_baseline"] = lif_cpu_sample(steps=6, images=nb, threads=t)
    return out


def lif_cpu_sample(steps=6, images=1, threads=1):
    """The same network through the oracle (its LIF update and presynaptic delivery, pinned to the
    reference's own loops): a bounded sample of `steps` timesteps for each of `images` images,
    one image per host thread."""
    from multiprocessing.pool import ThreadPool
    from oracle import oracle as O
    O.build()
    n, ne, ni = 256, 32, 8
    inp, exc, inh = O.Loc.make(1, n, n, 1, 5, 5), O.Loc.make(1, n, n, ne, 2, 2), O.Loc.make(1, n // 2, n // 2, ni, 2, 2)
    exc_r, inh_r = O.Loc.make(1, n, n, ne, 0, 0), O.Loc.make(1, n // 2, n // 2, ni, 0, 0)

    def gauss(nfpre, p, nfpost, sigma, peak):
        r = np.arange(p) - (p - 1) / 2.0
        g = np.exp(-(r[:, None] ** 2 + r[None, :] ** 2) / (2 * sigma ** 2))
        return np.ascontiguousarray(np.broadcast_to(peak * g[None, :, :, None], (nfpre, p, p, nfpost))).astype(np.float32)

    w_ie, w_ei, w_he = gauss(1, 11, ne, 3.0, 0.5), np.full((ne * 4, 3, 3, ni), 0.05, np.float32), gauss(ni, 8, ne, 2.0, 1.0)
    prm = O.lif_params_array()

    def state(loc, seed):
        m = loc.nx * loc.ny * loc.nf
        return {"rnd": O.taus_init(m, seed), "V": np.full(m, -70.0, np.float32), "Vth": np.full(m, -55.0, np.float32),
                "GE": np.zeros(m, np.float32), "GI": np.zeros(m, np.float32), "GIB": np.zeros(m, np.float32)}

    def run_image(i):
        rng = np.random.default_rng(1234 + 5 + i)
        se, sh = state(exc, 17 + 2 * i), state(inh, 18 + 2 * i)
        ae, ah = np.zeros(exc.ext_shape(), np.float32), np.zeros(inh.ext_shape(), np.float32)
        rates = rng.uniform(5, 50, (1, n, n, 1))
        for _ in range(steps):
            x = np.zeros(inp.ext_shape(), np.float32)
            x[:, 5:5 + n, 5:5 + n, :] = (rng.random((1, n, n, 1)) < rates * 1e-3).astype(np.float32)
            e, c = O.compact(x.reshape(1, -1))
            eh, ch = O.compact(ah.reshape(1, -1))
            g0 = O.deliver_pre(inp, exc_r, 11, 11, w_ie, entries=e, num_active=c)
            g1 = O.deliver_pre(inh, exc_r, 8, 8, w_he, entries=eh, num_active=ch)
            se, ae = O.lif_update("a", exc, prm, 1.0, se, np.stack([g0.reshape(-1), g1.reshape(-1), 0 * g0.reshape(-1)]),
                                  ae)
            ee, ce = O.compact(ae.reshape(1, -1))
            gi = O.deliver_pre(exc, inh_r, 3, 3, w_ei, entries=ee, num_active=ce).reshape(-1)
            sh, ah = O.lif_update("a", inh, prm, 1.0, sh, np.stack([gi, 0 * gi, 0 * gi]), ah)

    t0 = time.perf_counter()
    if threads > 1:
        with ThreadPool(threads) as pool:
            pool.map(run_image, range(images))
    else:
        for i in range(images):
            run_image(i)
    dt = time.perf_counter() - t0
    return {"value": images * steps / dt, "unit": "image-steps/s", "cores": threads, "kind": "port",
            "sample": f"oracle, the whole network for {images} image(s) x {steps} timesteps, one image per thread on "
                      f"{threads} host thread(s) ({dt:.2f} s)"}


# ---------------------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    cfg = dict(CFG)
    if args.timesteps:
        cfg["timesteps"] = args.timesteps
        cfg["x3_steps"] = min(cfg["x3_steps"], args.timesteps // 8)
    nb, T, X3 = cfg["nbatch"], cfg["timesteps"], cfg["x3_steps"]
    w_np, x_np = make_inputs(cfg, seed_offset=shard_seed_offset(rank))  # each rank solves its own batch shard
    vshape = (nb,) + cfg["v1_shape"]
    solver = capi.LcaSolver(nb, cfg["in_shape"], cfg["v1_shape"], cfg["nxp"], cfg["VThresh"], AMin=cfg["AMin"],
                            AShift=cfg["AShift"], VWidth=cfg["VWidth"], tau=cfg["tau"], dt=cfg["dt"])
    w = torch.from_numpy(w_np).to(dev)
    x = torch.from_numpy(x_np).to(dev)
    solver.set_weights(w)
    energy = torch.zeros(nb, dtype=torch.float64, device=dev)

    def solve(xd, precision=capi.LCA_BF16, x3=X3):
        solver.reset()
        solver.run(xd, T, x3_steps=x3, precision=precision)
        solver.energy(xd, energy)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # kernel shapes picked by the autotuner (timed with events on a few steps; outside the timed region)
    solver.autotune(x, trial_steps=4)
    tuned = solver.plan_info()
    tuned["schedule"] = solver.schedule()
    tuned["fused"] = solver.fused_plan_info()
    for _ in range(args.warmup):
        solve(x)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record()
        for _ in range(args.steps):
            solve(x)
        e1.record()
        torch.cuda.synchronize()
    barrier()
    # per-kernel split for the roofline: one more solve with CUDA events around every launch
    # (kernels launched one by one, no graph, no overlap between them); an NVTX range marks it
    # so that a profiler can select the tuned kernels of this solve (ncu --nvtx-include)
    solver.profile_begin(T)
    torch.cuda.nvtx.range_push("lca_profiled")
    solve(x)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    recon_ms, post_ms, fused_ms, nprof, nfused = solver.profile_end_fused()
    fused_shape = solver.fused_plan_info()
    ms = e0.elapsed_time(e1) / args.steps
    ms_all = max_over_ranks(ms, dist, dev)
    value = job_value(world, nb, T, ms_all)
    assert solver.error_flag() == 0, "a bounded device wait timed out"
    e_gpu = energy.cpu().numpy().copy()

    # end to end through the C ABI with host buffers: H2D input, solve, D2H activity + energy.
    # Step k's result is read back on a copy stream while step k+1 solves (two device result
    # buffers, two pinned host buffers); the timed region ends after the last step's read.
    x_host = torch.from_numpy(x_np).pin_memory()
    a_host = [torch.empty(vshape, dtype=torch.float32).pin_memory() for _ in range(2)]
    en_host = [torch.empty(nb, dtype=torch.float64).pin_memory() for _ in range(2)]
    x_dev = torch.empty_like(x)
    a_dev = [torch.empty(vshape, device=dev) for _ in range(2)]
    en_dev = [torch.empty(nb, dtype=torch.float64, device=dev) for _ in range(2)]
    main_stream, copy_stream = torch.cuda.current_stream(), torch.cuda.Stream()
    read_done = [None, None]

    def e2e_step(k):
        i = k & 1
        x_dev.copy_(x_host, non_blocking=True)
        solve(x_dev)
        if read_done[i] is not None:
            main_stream.wait_event(read_done[i])  # buffer i's previous read has finished
        solver.state(a=a_dev[i])
        en_dev[i].copy_(energy)
        copy_stream.wait_stream(main_stream)
        with torch.cuda.stream(copy_stream):
            a_host[i].copy_(a_dev[i], non_blocking=True)
            en_host[i].copy_(en_dev[i], non_blocking=True)
            read_done[i] = torch.cuda.Event()
            read_done[i].record(copy_stream)

    e2e_step(0)
    main_stream.wait_stream(copy_stream)
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for k in range(1, args.steps + 1):
        e2e_step(k)
    main_stream.wait_stream(copy_stream)
    t1.record()
    torch.cuda.synchronize()
    last = args.steps & 1
    solver.state(a=a_dev[last])
    torch.cuda.synchronize()
    assert torch.equal(a_host[last], a_dev[last].cpu()), "the last step's activity read back differs"
    assert torch.equal(en_host[last], energy.cpu()), "the last step's energies read back differ"
    e2e_ms = max_over_ranks(t0.elapsed_time(t1) / args.steps, dist, dev)
    e2e_value = job_value(world, nb, T, e2e_ms)
    h2d = x_np.nbytes
    d2h = a_host[0].numel() * 4 + nb * 8

    if rank != 0 or args.quick:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        if args.quick and rank == 0:
            print(json.dumps({"quick": True, "value": value, "ms_per_step": ms_all, "timesteps": T,
                              "recon_ms": recon_ms / max(nprof, 1), "post_ms": post_ms / max(nprof, 1),
                              "fused_ms_per_launch": fused_ms / max(nfused, 1), "fused_launches": nfused,
                              "fused_shape": fused_shape, "schedule": tuned["schedule"], "e2e_value": e2e_value}))
        return

    # plain FP32 form, same structure, no tensor cores
    solve(x, precision=capi.LCA_FP32, x3=0)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps32 = max(1, min(args.steps, 3))
    f0.record()
    for _ in range(reps32):
        solve(x, precision=capi.LCA_FP32, x3=0)
    f1.record()
    torch.cuda.synchronize()
    ms32 = f0.elapsed_time(f1) / reps32
    value32 = nb * T / (ms32 / 1000.0)
    e_fp32 = energy.cpu().numpy().copy()

    # final-energy error against the FP64 oracle on the first images
    nchk = int(os.environ.get("PVGPU_BENCH_FP64_IMAGES", "4"))
    cores = os.cpu_count() or 1
    e64 = fp64_energy(cfg, x_np, w_np, nchk, min(nchk, cores))
    rel_bf16 = float(np.max(np.abs(e_gpu[:nchk] - e64) / np.abs(e64)))
    rel_fp32 = float(np.max(np.abs(e_fp32[:nchk] - e64) / np.abs(e64)))

    # dominant kernel roofline: the fused timestep kernel F (or, with no fused steps, kernel P),
    # HBM-bound
    pk = peaks()
    npos, F = cfg["v1_shape"][0] * cfg["v1_shape"][1], cfg["v1_shape"][2]
    npix = int(np.prod(cfg["in_shape"]))
    mb = npos // 128
    x3_frac = X3 / T
    # per image-timestep, kernel P: V read + write (FP32), A written (BF16; + BF16 lo in BF16x3
    # steps), and the padded residual window of each (128-position, feature-tile) tile read once
    S = cfg["in_shape"][1] // cfg["v1_shape"][1]
    P, C = cfg["nxp"], cfg["in_shape"][2]
    E = (P - S) // 2
    rows_per_block = 128 // cfg["v1_shape"][1]
    RP = -(-(cfg["in_shape"][1] + 2 * E) * C // 4) * 4
    rows_pad = cfg["in_shape"][0] + 2 * E
    FT = min(F, 256)
    window_bytes = (S * (rows_per_block - 1) + P) * RP * 4
    # kernel P runs the BF16x3 steps and the run's last BF16 step when kernel F is on
    nP = nprof - nfused
    x3_frac_p = X3 / max(nP, 1)
    post_bytes_unit = npos * F * (4 + 4 + 2 + 2 * x3_frac_p) + mb * (F // FT) * window_bytes
    post_bytes_launch = post_bytes_unit * nb
    post_avg_ms = post_ms / max(nP, 1)
    # kernel F per image-timestep: V read + write (FP32); per (block, feature tile) tile the stage
    # (the block's bands of every feature tile + the P - S overlapping rows of each neighbour's)
    # read, its band written, and x on the rows the block owns read (feature tile 0)
    FTf = fused_shape["feature_tile"] or F
    nfh = F // FTf
    band = window_bytes
    slice_b = (P - S) * RP * 4
    stage = sum(nfh * band + ((mb_i > 0) + (mb_i < mb - 1)) * nfh * slice_b for mb_i in range(mb)) * nfh
    owned = sum(((S * (rows_per_block - 1) + P) if mb_i == mb - 1 else S * rows_per_block) * RP * 4
                for mb_i in range(mb))
    fused_bytes_unit = npos * F * 8 + stage + mb * nfh * band + owned
    fused_bytes_launch = fused_bytes_unit * nb
    fused_avg_ms = fused_ms / max(nfused, 1)
    if nfused:
        dom_name = "step_tc_kernel (fused timestep: post delivery GEMM, LCA update, reconstruction bands)"
        dom_bytes, dom_ms, dom_share = fused_bytes_launch, fused_avg_ms, fused_ms / (fused_ms + post_ms + recon_ms)
    else:
        dom_name = "post_tc_kernel (post delivery GEMM + LCA update, residual windows in)"
        dom_bytes, dom_ms, dom_share = post_bytes_launch, post_avg_ms, post_ms / (post_ms + recon_ms)
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    # kernel R: A read (BF16; + lo), x read, the padded residual written
    recon_bytes_unit = npos * F * (2 + 2 * x3_frac) + npix * 4 + rows_pad * RP * 4
    nR = nprof - nfused + (1 if nfused else 0)  # kernel R: every unfused step and the first fused one
    recon_avg_ms = recon_ms / max(nR, 1)
    recon_flops_launch = 2 * npos * F * (cfg["nxp"] ** 2 * cfg["in_shape"][2]) * nb * (1 + 2 * x3_frac)

    # DRAM bytes per launch from the committed ncu summary of the same kernel and workload
    traffic = None
    trafficf = os.path.join(ROOT, "profiles", ("step_tc_kernel_batched_lca.md" if nfused else
                                               "post_tc_kernel_batched_lca.md"))
    if os.path.exists(trafficf):
        for line in open(trafficf):
            if line.startswith("dram bytes per launch:"):
                traffic = float(line.split(":")[1])

    # kernels per solve: reset and energy, and per chain: x padded, kernel R + F on the first fused
    # step, F on the others, R + P on the rest (BF16x3 and the last BF16 step)
    chains = tuned["schedule"]["chains"]
    per_chain = (2 + nfused + 2 * (T - nfused)) if nfused else 2 * T
    launches_per_solve = 2 + chains * per_chain
    cpu_val, cpu_dt = cpu_sample(cfg, cores, warm_steps=25, timed_steps=25)
    deliv = delivery_bench(torch, capi)
    c1b = config1_bench(torch, capi)
    lifb = lif_bench(torch, capi)
    dlb = dictlearn_bench(torch, capi)
    clocks = clk.summary()

    # the FP32 form against its own ceiling: FP32 FMA lanes x 2 FLOP x SM clock (nominal lanes,
    # sampled clock), on 4 x 25,165,824 FLOP per image-timestep (post delivery + reconstruction)
    props = torch.cuda.get_device_properties(0)
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    fp32_peak_tflops = props.multi_processor_count * 128 * 2 * sm_mhz * 1e6 / 1e12
    flop_unit = 4 * npos * F * cfg["nxp"] ** 2 * cfg["in_shape"][2]
    fp32_tflops = value32 * flop_unit / 1e12
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "images*steps/s",
        "final_energy_rel_err_vs_fp64": rel_bf16,
        "speedup_bf16_over_fp32_form": value / world / value32,
        # against an FP32 form running at its FMA ceiling (the same FLOPs at fp32_fma_ceiling_tflops)
        "speedup_bf16_over_fp32_fma_ceiling": value / world / (fp32_peak_tflops * 1e12 / flop_unit),
        "fp32_form": {"value": value32, "unit": "images*steps/s", "final_energy_rel_err_vs_fp64": rel_fp32,
                      "TFLOP_s": fp32_tflops, "fp32_fma_ceiling_tflops": fp32_peak_tflops,
                      "frac_of_fp32_fma_ceiling": fp32_tflops / fp32_peak_tflops},
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_all,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16",
        "data": "synthetic",
        "config": {"workload": "batched LCA: 256 images 32x32x3 (1/f, unit std) -> V1 16x16x512 stride 2, "
                               "dictionary 512 x 8x8x3, VThresh=AShift=0.15, tau=100, 400 timesteps, BF16x3 last 50",
                   "global_batch": nb * world, "timesteps_per_step": T, "parallelism": f"replicas{world}",
                   "l2": "state streamed each timestep (V 134 MB + activity 67 MB per step > 129 MB L2)",
                   "kernel_shapes": tuned},
        "gpu_launches": args.steps * launches_per_solve,
        "e2e": {"value": e2e_value, "unit": "images*steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "read_back": "each step's activity and energies, on a copy stream during the next step's solve"},
        "roofline": {"bound": "hbm", "kernel": dom_name,
                     "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                     "peak_source": pk["source"], "traffic": traffic, "bytes_per_launch": dom_bytes,
                     "avg_launch_ms": dom_ms, "share_of_step": dom_share, "launches_per_solve": nfused or nprof},
        "post_kernel": {"avg_launch_ms": post_avg_ms, "launches_per_solve": nP,
                        "GB_s": post_bytes_launch / (post_avg_ms / 1e3) / 1e9 if nP else None},
        "recon_kernel": {"avg_launch_ms": recon_avg_ms, "GB_s": recon_bytes_unit * nb / (recon_avg_ms / 1e3) / 1e9,
                         "TFLOP_s": recon_flops_launch / (recon_avg_ms / 1e3) / 1e12},
        "energy_check_images": nchk,
        "cpu_baseline": {"value": cpu_val, "unit": "images*steps/s", "cores": cores, "kind": "port",
                         "sample": f"oracle FP32 LCA, {cores} images (one per thread) x 25 timesteps after 25 "
                                   f"warm-up timesteps, same layer sizes ({cpu_dt:.1f} s)"},
        "delivery": {"workload": "delivery 16 x (128x128x256 -> 128x128x64), 7x7 shared weights: presynaptic "
                                 "sparse (SparseList) and tensor-core (dense activity, split-TF32) at three "
                                 "densities; postsynaptic FP32 SIMT and tensor-core",
                     "by_density": {k: v for k, v in deliv.items() if k != "post"}, "post": deliv["post"],
                     "hbm_peak_gbs": pk["hbm_gbs"], "tf32_tensor_peak_tflops": pk["bf16_tflops"] / 2},
        "plain_lca_batch1": c1b,
        "lif_network": lifb,
        "dictionary_learning": dlb,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=12)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--timesteps", type=int, default=0, help="override the 400 LCA timesteps (profiling runs)")
    ap.add_argument("--quick", action="store_true", help="time the solve only (profiling runs; not a bench line)")
    ap.add_argument("--delivery", action="store_true",
                    help="run the presynaptic delivery microbenchmark only (profiling runs; not a bench line)")
    ap.add_argument("--lif", action="store_true",
                    help="run the LIF network only (profiling runs; not a bench line)")
    ap.add_argument("--lif-steps", type=int, default=1000, help="timesteps of the LIF network graph (--lif)")
    ap.add_argument("--dictlearn", action="store_true",
                    help="run the dictionary-learning gradient section only (profiling runs; not a bench line)")
    ap.add_argument("--plain-lca", action="store_true",
                    help="run the batch-1 plain LCA latency section only (profiling runs; not a bench line)")
    args = ap.parse_args()
    if args.dictlearn:
        import torch
        from openpv_gb300 import build
        build.build()
        from openpv_gb300 import capi
        print(json.dumps({"dictionary_learning": dictlearn_bench(torch, capi)}))
        return
    if args.plain_lca:
        import torch
        from openpv_gb300 import build
        build.build()
        from openpv_gb300 import capi
        print(json.dumps({"plain_lca_batch1": config1_bench(torch, capi, reps=1)}))
        return
    if args.lif:
        import torch
        from openpv_gb300 import build
        build.build()
        from openpv_gb300 import capi
        print(json.dumps({"lif_network": lif_bench(torch, capi, steps=args.lif_steps, cpu_sample=False)}))
        return
    if args.delivery:
        import torch
        from openpv_gb300 import build
        build.build()
        from openpv_gb300 import capi
        print(json.dumps({"delivery": delivery_bench(torch, capi, reps=1)}))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.impl == "ours" else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus and "WORLD_SIZE" not in os.environ:
        world = 1
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
