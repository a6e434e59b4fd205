"""Benchmark: D3Q27 RR lattice updates per second on one GB300.

Workload (the configuration the headline metric is quoted on): lid-driven
cavity, 128^3, D3Q27 RR, Re = 1000, lid 0.1 in +x on the top (y-hi) wall,
half-way bounce-back on all six faces, FP16 shifted-population storage with
FP32 arithmetic.  One "step" = one fused time step over the whole grid.

Line fields (one JSON line on rank 0):
  value      MLUPS over the timed steps, each step timed alone with CUDA
             events on the solver's stream, L2 flushed before every timed
             step (a 256 MB write, then a 256 MB read of a second buffer so
             that the write's dirty lines leave L2 before the step); inputs
             resident in HBM.
  e2e        the same metric through the C ABI with host buffers: upload of
             the start state from pinned host memory (rr_init_state), the K
             steps, and the macroscopic fields read back to the host
             (rr_macro), all inside the timed region.
  roofline   the step kernel against the measured HBM copy bandwidth:
             algorithmic bytes = 27 populations x 2 B read + written = 108 B
             per lattice update.
  cpu_baseline  the oracle (C restatement of the reference step, OpenMP on
             all host threads) on a bounded sample of the same workload;
             cpu_baseline_1core the same on one thread (the reference's CPU
             programs are serial).
  batch      the multi-domain form: 256 seeded Taylor-Green / cavity domains
             (FP16 storage) advanced by one persistent launch per step inside
             CUDA graphs, against the same domains stepped one at a time
             (each domain's own rr_step, synchronised) and on concurrent
             per-domain streams; aggregate MLUPS over a fixed step count.
  serving    the served form: seeded Poisson streams of Taylor-Green, cavity
             and WALE channel solves (the mixed stream: 32^3-192^3, 1k-20k
             steps at 200 req/s; the small-solve stream: 32^3-64^3, 1k-4k
             steps at 400 req/s) through the continuous-batching server under
             an 80 GB budget, against a one-at-a-time server; solves/s,
             p50/p99 latency (overall, per size class, queueing and device
             parts) and each sampled solve's velocity error against its FP64
             rerun.
--impl reference runs that CPU implementation alone as the reference arm.
Multi-GPU (torchrun, N > 1): independent replicas, one domain per GPU.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "recursively-regularized-lbm_gb300"))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "cavity128_f16": dict(kind="cavity", n=128, storage="f16", Re=1000.0, U=0.1),
    "cavity128_f32": dict(kind="cavity", n=128, storage="f32", Re=1000.0, U=0.1),
    "cavity128_f64": dict(kind="cavity", n=128, storage="f64", Re=1000.0, U=0.1),
    "cavity128_bf16": dict(kind="cavity", n=128, storage="bf16", Re=1000.0, U=0.1),
    "channel_les_f16": dict(kind="channel", storage="f16"),
    "channel_les_f32": dict(kind="channel", storage="f32"),
    "channel_les_f64": dict(kind="channel", storage="f64"),
    "channel_dns_f16": dict(kind="channel", storage="f16", les=False),
    "channel_fdbc_f16": dict(kind="channel", storage="f16", les=False, fdbc=True),
    "channel_les_fdbc_f16": dict(kind="channel", storage="f16", fdbc=True),
    "tg100_f64": dict(kind="tg", storage="f64"),
    "tg128_f16": dict(kind="tg128", storage="f16"),
    "tg128_f32": dict(kind="tg128", storage="f32"),
    "tg128_bgk_f16": dict(kind="tg128", storage="f16", bgk=True),
}
BYTES_PER_POP = {"f64": 8, "f32": 4, "f16": 2, "bf16": 2}
DTYPE = {"f64": "f64", "f32": "f32", "f16": "f16-store/f32-compute", "bf16": "bf16-store/f32-compute"}


def make(wl):
    from rrlbm import presets
    w = WORKLOADS[wl]
    if w["kind"] == "cavity":
        return presets.cavity(n=w["n"], Re=w["Re"], U=w["U"], storage=w["storage"], variant="config")
    if w["kind"] == "channel":
        p, st = presets.channel(storage=w["storage"], les=w.get("les", True), variant="config")
        if w.get("fdbc"):
            import rrlbm
            p.face[2] = p.face[3] = rrlbm.FACE_FDBC
        return p, st
    if w["kind"] == "tg128":
        p, st = presets.taylor_green(L=128, nz=128, tau=0.6, Ma=0.05, storage=w["storage"])
        if w.get("bgk"):
            import rrlbm
            p.collision = rrlbm.COLL_BGK
            st["f"] = None  # the BGK run starts from the second-order equilibrium of the fields
        return p, st
    return presets.taylor_green(L=100, nz=4, tau=0.6, Ma=0.01, storage=w["storage"])


def describe(wl, p):
    """the workload, the same string on both arms (the storage type is the
    line's dtype)"""
    kind = WORKLOADS[wl]["kind"]
    if kind == "cavity":
        return (f"lid-driven cavity {p.lx}x{p.ly}x{p.lz} D3Q27 RR, Re=1000, lid 0.1 +x on y-hi, "
                f"bounce-back + regularized closure on 6 faces")
    if kind == "channel":
        w = WORKLOADS[wl]
        model = "RR + WALE (C_w=0.5)" if w.get("les", True) else "RR DNS"
        walls = "finite-difference closure (FDBC)" if w.get("fdbc") else "bounce-back + regularized closure"
        return (f"channel {p.lx}x{p.ly}x{p.lz} D3Q27 {model}, Re_tau=180, walls y ({walls}), periodic x/z, "
                f"body force")
    ma = 0.05 if kind == "tg128" else 0.01
    coll = "BGK" if WORKLOADS[wl].get("bgk") else "RR"
    return f"Taylor-Green {p.lx}x{p.ly}x{p.lz} D3Q27 {coll}, Ma={ma}, tau=0.6, periodic"


def config_of(wl, p, world):
    """the line's config, identical on the GPU arm and the reference arm"""
    return {"workload": describe(wl, p), "nodes": p.n, "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: flushed before every timed step (256 MB write, then 256 MB read of a second "
                  "buffer); the CPU arm has no flush"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic(wl):
    """DRAM bytes per step-kernel launch from the committed ncu summary, if any"""
    path = os.path.join(ROOT, "profiles", f"tile_kernel_{wl}.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi samples during the timed region"""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap,utilization.gpu")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                util = float(s[7])
                if util > 0:
                    sm.append(float(s[0]))
                mx = max(mx, float(s[1]))
                for k, v in zip(names, s[3:7]):
                    if v.lower() == "active":
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        if not sm:
            sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def cpu_baseline(wl, budget_s, cores=None):
    """the oracle on the machine's host cores (all of them by default), on whole
    steps of the workload"""
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import load_state, oracle_for
    p, st = make(wl)
    cores = cores or os.cpu_count() or 1
    O.set_threads(cores)
    o = oracle_for(p)
    load_state(o, st)
    o.run(1)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        o.run(1)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s:
            break
    O.set_threads(os.cpu_count() or 1)
    mlups = p.n * steps / el / 1e6
    how = f"OpenMP over {cores} threads" if cores > 1 else "one thread"
    return {"value": mlups, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{steps} full steps of the {p.lx}x{p.ly}x{p.lz} workload in FP64 "
                      f"({el:.1f} s), {how}"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    K, W = args.steps, args.warmup
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import load_state, oracle_for
    p, st = make(args.workload)
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o = oracle_for(p)
    load_state(o, st)
    t0 = time.perf_counter()
    o.run(max(W, 1))
    per_step = (time.perf_counter() - t0) / max(W, 1)
    # a bounded sample: at most about two minutes of host work
    Ks = max(1, min(K, int(120.0 / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    o.run(Ks)
    el = time.perf_counter() - t0
    v = p.n * Ks / el / 1e6
    line = {"metric": "D3Q27 RR MLUPS (lattice updates per second)", "value": v, "unit": "MLUPS",
            "impl": "reference", "n_gpus": args.gpus, "steps": K, "warmup": W,
            "ms_per_step": el / Ks * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(args.workload, p, world),
            "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": cores, "kind": "port",
                             "sample": f"{Ks} of the {K} requested full steps (at most ~2 min of host work) after "
                                       f"{max(W, 1)} warm-up steps, OpenMP over {cores} threads"},
            "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(x, dist):
    """the maximum of a per-rank float over all ranks (NCCL on the GPU, gloo
    on the host)"""
    if not dist:
        return x
    import torch
    import torch.distributed as tdist
    dev = "cuda" if tdist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def set_dns(s, how):
    """the DNS step's method: tile (one launch of warp items), staged (shared-
    memory pipeline of bulk copies) or tuned by rr_tune's choice for the class"""
    if how == "tile":
        s.set_stage(0)
    elif how == "staged":
        s.set_stage(1)


def run_gpu(args, rank, world, local_rank):
    import numpy as np
    import torch
    import rrlbm

    K, W = args.steps, args.warmup
    torch.cuda.set_device(local_rank)
    p, st = make(args.workload)
    p.device = local_rank
    storage = WORKLOADS[args.workload]["storage"]
    q = p.q
    n = p.n
    dist = world > 1
    if dist:
        import torch.distributed as tdist

    s = rrlbm.Solver(p)
    set_dns(s, args.dns)
    # rr kernel launches per step: tile step 1; staged step 2 (interior +
    # face rows); WALE two-pass 2, fused 1; the finite-difference closure one
    # more per pass
    les_method, dns_method = s.launch()[1], s.stage()[0]
    launches_per_step = (2 if les_method == 1 else 1) if p.use_les else (2 if dns_method == 1 else 1)
    if rrlbm.FACE_FDBC in (p.face[2], p.face[3]):
        launches_per_step += 2 if p.use_les else 1
    s.init_state(st["rho"], st["ux"], st["uy"], st["uz"], f=st.get("f"))
    stream = torch.cuda.ExternalStream(s.stream)
    # L2 flush before every timed step: a 256 MB write, then a 256 MB read of
    # a second buffer, whose clean lines evict the write's dirty ones (their
    # write-back happens here, not inside the next timed step)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    flush_rd = torch.ones(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sink = torch.empty((), dtype=torch.float32, device="cuda")
    # warm-up (also builds nothing lazily on the timed path)
    s.step(W)
    s.sync()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    with Clocks(local_rank) as clk:
        # hold the stream behind a bounded spin (about 40 ms) while the host
        # enqueues all K iterations, so host launch latency never lands
        # inside a timed window
        with torch.cuda.stream(stream):
            torch.cuda._sleep(int(4e7 + 5e4 * K))
        for k in range(K):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))  # evict the populations from L2
                torch.sum(flush_rd, dim=0, out=sink)
                evs[k][0].record(stream)
            s.step(1)
            with torch.cuda.stream(stream):
                evs[k][1].record(stream)
        s.sync()
        torch.cuda.synchronize()
    times = [a.elapsed_time(b) for a, b in evs]  # ms
    t_step = sum(times) / K
    t_step = max_over_ranks(t_step, dist)
    value = n * world / (t_step * 1e-3) / 1e6

    if args.no_e2e:
        s.close()
        if rank == 0:
            line = {"value": value, "unit": "MLUPS", "ms_per_step": t_step, "workload": args.workload,
                    "note": "profiling run, no e2e"}
            if world == 1 and args.batch_steps > 0:
                line["batch"] = run_batch(args)
            print(json.dumps(line), flush=True)
        return
    # end to end through the C ABI with host buffers
    pin = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory() for k in ("rho", "ux", "uy", "uz")}
    outs = {k: torch.empty((n,), dtype=torch.float64).pin_memory() for k in ("rho", "ux", "uy", "uz")}
    s2 = rrlbm.Solver(p)
    set_dns(s2, args.dns)
    arr = {k: pin[k].numpy() for k in pin}
    s2.init_state(arr["rho"], arr["ux"], arr["uy"], arr["uz"])
    s2.step(W)
    s2.sync()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s2.init_state(arr["rho"], arr["ux"], arr["uy"], arr["uz"])
    s2.step(K)
    s2.macro_into(*(outs[k].numpy().reshape(p.shape) for k in ("rho", "ux", "uy", "uz")))
    e2e_t = time.perf_counter() - t0
    e2e_t = max_over_ranks(e2e_t, dist)
    e2e = n * K * world / e2e_t / 1e6
    assert np.isfinite(outs["ux"].numpy()).all()
    s2.close()
    s.close()
    if rank != 0:
        return
    pk, src = peaks()
    bpl = 2 * q * BYTES_PER_POP[storage]
    achieved = n * bpl / (t_step * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload)
    line = {
        "metric": "D3Q27 RR MLUPS (lattice updates per second)", "value": value, "unit": "MLUPS",
        "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[storage], "data": "synthetic",
        "config": config_of(args.workload, p, world),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                     "bytes_per_lup": bpl, "peak_source": f"{src} (hbm_gbs)"},
        "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": 4 * 8 * n / K,
                "d2h_bytes_per_step": 4 * 8 * n / K,
                "what": "rr_init_state from pinned host arrays + K steps + rr_macro to pinned host arrays"},
        "gpu_launches": K * launches_per_step,
        "clocks": clk.summary(),
        "step_ms_min": min(times), "step_ms_max": max(times),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_seconds)
        # the reference's CPU programs are serial: the like-for-like line
        line["cpu_baseline_1core"] = cpu_baseline(args.workload, args.cpu_seconds / 2, cores=1)
    if world == 1 and args.batch_steps > 0:
        # the batch section's own timed region keeps its own launch count
        line["batch"] = run_batch(args)
    if world == 1 and args.serve_requests > 0:
        line["serving"] = run_serve(args)
    print(json.dumps(line), flush=True)


def run_batch(args):
    """The multi-domain form: aggregate MLUPS of one batch against per-domain
    launches, same domains, same step count."""
    import torch
    import rrlbm
    from rrlbm import workloads

    K = args.batch_steps
    doms = workloads.ensemble(args.batch_domains, steps=K)
    solvers = []
    for d in doms:
        s = rrlbm.Solver(workloads.params_of(d))
        rho, ux, uy, uz = workloads.macros_on_device(d)
        s.init_state(rho, ux, uy, uz)
        s.sync()
        solvers.append(s)
    nodes = sum(d.nodes for d in doms)
    out = {"domains": len(doms), "steps": K, "nodes": nodes, "storage": "f16",
           "mix": "seeded: Taylor-Green cubes 32^3-128^3 (Ma 0.01-0.1, tau 0.52-0.8), "
                  "cavities 32^3-96^3 (Re 100-1000), log-uniform sizes"}
    # one at a time: each domain's own rr_step(K) (graphs of 32 steps), synchronised
    for s in solvers:
        s.step(2)
        s.sync()
    t0 = time.perf_counter()
    for s in solvers:
        s.step(K)
        s.sync()
    t_seq = time.perf_counter() - t0
    # per-domain launches on concurrent streams
    t0 = time.perf_counter()
    for s in solvers:
        s.step(K)
    for s in solvers:
        s.sync()
    t_conc = time.perf_counter() - t0
    # the batch: tuned launch shapes, then K steps timed on its stream
    b = rrlbm.Batch()
    for s in solvers:
        b.add(s)
    tune_steps = b.tune(trial_steps=8)
    st = torch.cuda.ExternalStream(b.stream)

    def timed():
        b.step(2 * 32)
        b.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(st)
        b.step(K)
        e1.record(st)
        b.sync()
        return time.perf_counter() - t0, e0.elapsed_time(e1) * 1e-3

    mode, chains = b.mode()
    block, cps, order = b.launch()
    t_batch, t_dev = timed()
    # the other mode, for the record
    b.set_mode(1 - mode, chains)
    t_other, _ = timed()
    b.set_mode(mode, chains)
    grouping = b.grouping
    b.close()
    for s in solvers:
        s.close()
    mlups = lambda t: nodes * K / t / 1e6
    out.update({
        "mlups": mlups(t_batch), "mlups_device": mlups(t_dev),
        "mlups_one_at_a_time": mlups(t_seq), "mlups_concurrent_streams": mlups(t_conc),
        "speedup_vs_one_at_a_time": t_seq / t_batch, "speedup_vs_concurrent_streams": t_conc / t_batch,
        "mode": ["persistent kernel", "fan-out of member launches"][mode],
        f"mlups_{['fanout', 'persistent'][mode]}": mlups(t_other),
        "tuned": {"mode": mode, "chains": chains, "block": block, "ctas_per_sm": cps,
                  "order": ["strided", "chunked"][order], "grouping_bytes": grouping, "tuning_steps": tune_steps},
        # persistent: one launch per step and class (a single storage/lattice class here);
        # fan-out: every member's own launch per step
        "launches": K if mode == 0 else K * len(doms),
    })
    return out


SERVE_STREAMS = {
    # the served workload: Taylor-Green / cavity / WALE channel, n^3 with n in
    # [32, 192] and steps in [1000, 20000] log-uniform, Poisson 200 req/s
    "mixed": dict(rate=200.0, seed=5, sizes=(32, 192), steps=(1000, 20000), scale=1),
    # small solves dominate: n in [32, 64], steps in [1000, 4000], Poisson
    # 400 req/s, five times the requests (a rate one domain at a time cannot
    # keep up with: its small grids leave the GPU mostly idle)
    "small": dict(rate=400.0, seed=9, sizes=(32, 64), steps=(1000, 4000), scale=5),
}


def serve_stream(name, count):
    from rrlbm import workloads
    c = SERVE_STREAMS[name]
    return workloads.request_stream(count * c["scale"], rate=c["rate"], seed=c["seed"], sizes=c["sizes"],
                                    steps=c["steps"])


def run_serve(args):
    """The served form: continuous batching against one-at-a-time serving on
    the same seeded request streams, and sampled errors against FP64 reruns."""
    import numpy as np
    from rrlbm import serve, workloads

    budget = 80e9
    out = {"budget_bytes": budget}
    for name in SERVE_STREAMS:
        reqs = serve_stream(name, args.serve_requests)
        c = SERVE_STREAMS[name]
        o = {"requests": len(reqs), "rate_per_s": c["rate"], "seed": c["seed"],
             "mix": f"Poisson arrivals; Taylor-Green / cavity / WALE channel; n^3 with n in "
                    f"[{c['sizes'][0]}, {c['sizes'][1]}] and steps in [{c['steps'][0]}, {c['steps'][1]}] "
                    f"log-uniform; FP16 or FP32 storage, FP32 compute"}
        for mode, slots in (("batched", None), ("one_at_a_time", 1)):
            be = serve.GpuBackend()
            # each solve's result: its domain means (rr_diag), read before it leaves
            srv = serve.Server(be, budget, max_active=slots, on_result=lambda s: s.diag())
            recs = srv.run(reqs)
            be.close()
            st = serve.summarize(recs)
            st["chunks"] = srv.chunks
            st["peak_resident"] = srv.peak_active
            st["peak_bytes"] = srv.peak_bytes
            o[mode] = st
        o["speedup_solves_per_s"] = o["batched"]["solves_per_s"] / o["one_at_a_time"]["solves_per_s"]
        out[name] = o
    # errors against FP64 reruns, sampled solves of the mixed stream (served
    # arithmetic = alone arithmetic, bit for bit, so the served result is the
    # alone run): the smallest by work, up to ~2e10 updates
    reqs = serve_stream("mixed", args.serve_requests)
    order = sorted(reqs, key=lambda d: d.nodes * d.steps)
    sample, work = set(), 0.0
    for d in order:
        if work + d.nodes * d.steps > 2e10 or len(sample) >= 8:
            break
        sample.add(d.rid)
        work += d.nodes * d.steps
    errs = []
    for d in reqs:
        if d.rid not in sample:
            continue
        lo, hi = workloads.solve_alone(d), workloads.solve_alone(d, "f64")
        a, b = lo.macro(), hi.macro()
        lo.close()
        hi.close()
        u = workloads.velocity_scale(d)
        e_max = max(float(np.abs(a[k] - b[k]).max()) for k in ("ux", "uy", "uz")) / u
        num = sum(float(((a[k] - b[k]) ** 2).sum()) for k in ("ux", "uy", "uz"))
        den = sum(float((b[k] ** 2).sum()) for k in ("ux", "uy", "uz"))
        errs.append({"rid": d.rid, "kind": d.kind, "n": d.n, "steps": d.steps, "storage": d.storage,
                     "max_err_rel_u": e_max, "l2_rel": (num / den) ** 0.5 if den > 0 else None})
    out["fp64_rerun_errors"] = errs
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cavity128_f16", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="device-timed steps only (profiling runs)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--dns", default="tile", choices=["tile", "staged"],
                    help="DNS step method of the single-domain lines (results are the same bit for bit)")
    ap.add_argument("--batch-domains", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=1000, help="0: skip the multi-domain line")
    ap.add_argument("--serve-requests", type=int, default=32, help="0: skip the serving line")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    try:
        run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as tdist
            tdist.destroy_process_group()


if __name__ == "__main__":
    main()
