#!/usr/bin/env python3
"""WHIR commit+open proofs per second on GB300.

A step is one complete WHIR proof of the plain single-instance workload:
commit + open of a seeded 2^24-evaluation KoalaBear multilinear polynomial,
rate 1/4 (log_inv_rate 2), folding factor 4, initial_reduction 1,
JohnsonBound at 100-bit security, 4 evaluation claims drawn from the
transcript as the reference harness draws them (crates/whir/src/test.rs:174-254).

  value   proofs/s with the polynomial already resident in HBM
  e2e     proofs/s through the C ABI from a pinned host buffer: the
          polynomial's host->device copy and every device->host read of the
          proof (roots, evaluations, openings, round messages) are inside the
          timed region
  roofline   the dominant kernel class, timed with CUDA events on the
          library's stream during the timed region
  cpu_baseline   the C restatement of the reference prover (oracle/) on the
          host cores, same workload, bounded sample

`--impl reference` times the reference's algorithm on the host CPU: the
reference (Rust) cannot be built in this environment, so its C restatement in
oracle/ runs with all host threads on the same workload.

Multi-GPU: proofs are independent, so N GPUs run N replicas (weak scaling);
value = proofs of all ranks / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(k=24, folding=4, rate=2, initial_reduction=1, soundness="JohnsonBound",
                soundness_id=1, security_level=100, claims=4, seed=1)
METRIC = "proofs/sec and p50/p99 latency, batched/served vs plain, 1 GB300, bit-exact"
UNIT = "proofs/s"
# Per-launch DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of the
# kernel classes, from one ncu capture of a full k = 24 proof (the five
# leaf-hash launches: 1473.0 MB per proof / 5 launches); the capture, its
# command and the per-launch figures are kept with the ncu summaries (profiles/).
NCU_TRAFFIC_BYTES = {"leaf_hash": 294.6e6}
NCU_TRAFFIC_K = 24
# Thread instructions per width-24 permutation of the leaf hash
# (smsp__inst_executed.sum * 32 / permutations of hash_rows_fixed<16> on a
# k = 22 proof, the ncu summary of the leaf hash in profiles/).  With one warp
# instruction issued per cycle on each of the 4 sub-partitions of each SM,
# the issue-bound rate is SMs * 4 * 32 * clock / this.
LEAF_INSTR_PER_PERM24 = 8087
GB300_SMS = 152


def leaf_permutations(k, folding, rate, initial_reduction):
    """Width-24 permutations of the leaf hashing of one proof: one per base
    codeword row, 4 per extension row (64 words), over the commitments of
    Whir::open's rounds (the round shapes of crates/whir/src/whir.rs:150-166)."""
    perms = 1 << (k + rate - folding)
    if k <= 6:
        return perms
    nr = (k - 6 + folding - 1) // folding
    for r in range(nr - 1):
        this_red = initial_reduction + r
        this_rate = rate + (r + 1) * folding - this_red
        kp = k - folding * (r + 1)
        perms += 4 * (1 << (kp + this_rate - folding))
    return perms


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--k", type=int, default=WORKLOAD["k"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="time budget of the bounded CPU baseline sample")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch splits (profiling runs)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched / served workloads")
    ap.add_argument("--workers", type=int, default=0,
                    help="concurrent provers of the batched / served runs (0: from host cores)")
    ap.add_argument("--serve-jobs", type=int, default=400,
                    help="requests per arrival rate of the served Poisson streams")
    ap.add_argument("--no-whir-bench-shape", action="store_true",
                    help="skip the reference's benchmark shapes (whir_bench, Merkle benches)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return world, rank, local


def max_over_ranks(x, world, device):
    """The largest x over all ranks (the slowest replica's time); x on one rank."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, slowest_s):
    """Whole-job proofs/s of N independent replicas: every rank proves
    `steps` proofs, the job ends with the slowest rank (weak scaling)."""
    return world * steps / slowest_s


# Structural instruction count of one Poseidon2 permutation: the operations
# its definition requires, each at the fewest 32-bit instructions it can take
# on the SM (31-bit p leaves no headroom for lazy sums in a 32-bit word):
#   Montgomery product: 64-bit product, t = lo * p^-1, high half of t p, subtract  4
#   modular add or subtract of canonical words: sum, sum - p, unsigned min         3
#   S-box x^3 of (x + rc): the add, two products, the canonical correction       11
#   light MDS (width 4c): mat4 = 9 adds + 2 doublings per group, 4 column sums
#     of c terms, one final add per lane
#   internal layer: S-box on lane 0; the lane sum in 64 bits (pairs in 32 bits,
#     then carried adds, one fold of 2^31 = 2^24 - 1 and a correction); per lane
#     sum + d x: |d| = 1: one modular op; |d| = 2: doubling + add; |d| = 3, 4:
#     a 64-bit multiply-add and its reduction (7); d = +-2^-e: shift, mask,
#     multiply-add, add and correction (6)
P2_STRUCTURE = {
    24: {"rounds_p": 23,
         "diag": [-2, 1, 2, .5, 3, 4, -.5, -3, -4] + [2 ** -e for e in (8, 2, 3, 4, 5, 6, 24)]
                 + [-2 ** -e for e in (8, 3, 4, 5, 6, 7, 9, 24)]},
}


def p2_structural_instructions(width):
    """Fewest 32-bit instructions one width-`width` permutation can take under
    the operation costs above (8 external rounds, the initial light MDS)."""
    st = P2_STRUCTURE[width]
    prod, modop, sbox = 4, 3, 11
    c = width // 4
    mds = modop * (11 * c + 4 * (c - 1) + width)
    lane = {1: modop, 2: 2 * modop, 3: 7, 4: 7}
    lanes = sum(lane[int(abs(d))] if abs(d) >= 1 else 6 for d in st["diag"])
    lane_sum = width // 2 + (width // 2 - 1) + 3 + 2
    internal = sbox + lane_sum + lanes
    assert prod * 2 + 3 == sbox
    return 8 * width * sbox + 9 * mds + st["rounds_p"] * internal


def integer_roofline(k, prof, clk):
    """The leaf hash against the integer issue rate: achieved width-24
    permutations/s over SMs * 4 * 32 * SM clock / instructions per
    permutation, with the fewer of the structural count and the kernel's
    measured count (the tighter bound)."""
    ms = prof["leaf_hash"]["ms_per_step"]
    if not ms:
        return None
    perms = leaf_permutations(k, WORKLOAD["folding"], WORKLOAD["rate"],
                              WORKLOAD["initial_reduction"])
    achieved = perms / (ms * 1e-3)
    mhz = clk.get("sm_mhz") or 2070.0
    structural = p2_structural_instructions(24)
    instr = min(structural, LEAF_INSTR_PER_PERM24)
    peak = GB300_SMS * 4 * 32 * mhz * 1e6 / instr
    return {"kernel": "leaf_hash", "bound": "integer issue", "unit": "perm24/s",
            "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "structural_instructions_per_perm24": structural,
            "kernel_instructions_per_perm24": LEAF_INSTR_PER_PERM24,
            "peak_source": f"{instr} instructions per permutation (the fewer of the structural "
                           f"count and the kernel's, ncu) at {mhz:.0f} MHz, 152 SMs x 4 issue "
                           f"slots of 32 lanes",
            "note": "the kernel issues fewer instructions than the structural count; the gap "
                    "to the issue rate is pipe contention (FMA-heavy 87%, ALU 67%, profiles/)"}


def workload_config(k):
    return {
        "workload": f"WHIR commit+open, 2^{k} KoalaBear evaluations, rate 1/4, folding 4, "
                    f"{WORKLOAD['claims']} claims, JohnsonBound 100-bit, initial_reduction 1",
        "k": k, "log_inv_rate": WORKLOAD["rate"], "folding": WORKLOAD["folding"],
        "initial_reduction": WORKLOAD["initial_reduction"], "soundness": WORKLOAD["soundness"],
        "security_level": WORKLOAD["security_level"], "claims": WORKLOAD["claims"],
        "seed": WORKLOAD["seed"], "field": "KoalaBear + degree-4 extension",
        "hash": "Poseidon2 (width-24 leaf sponge, width-16 compression)",
        "l2": "no flush needed: each step touches > 2 GB (codewords + trees) >> 129 MB L2",
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms (the timed
    region of the default run lasts about 0.3 s)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(k, seconds, expect_proof=None):
    """Oracle (C restatement, OpenMP over all host cores) on the same workload."""
    from oracle import oracle as O
    params = (k, WORKLOAD["folding"], WORKLOAD["rate"], WORKLOAD["initial_reduction"],
              WORKLOAD["soundness_id"], WORKLOAD["security_level"])
    poly = O.rand_fe(WORKLOAD["seed"], 1 << k)
    groups = [[0]] * WORKLOAD["claims"]
    n, t0 = 0, time.perf_counter()
    proof = None
    O.set_packed(True)  # Merkle hashing lane-packed, as the reference's packed Poseidon2
    try:
        while True:
            proof, _ = O.prove(params, [poly], [k], groups)
            n += 1
            el = time.perf_counter() - t0
            if el >= seconds or el * (n + 1) / n > 30.0:
                break
    finally:
        O.set_packed(False)
    same = None if expect_proof is None else bool(proof == expect_proof)
    return {"value": n / el, "unit": UNIT, "cores": O.lib().wo_threads(), "kind": "port",
            "sample": f"{n} full proofs of the same 2^{k} workload in {el:.1f} s "
                      f"(oracle/: C restatement of the reference prover, OpenMP over the host "
                      f"cores; Merkle leaves and nodes hashed {8} states per call through the "
                      f"lane-packed permutation the compiler vectorises, as the reference's "
                      f"packed Poseidon2 does)",
            "gpu_proof_identical": same}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    k = args.k
    params = (k, WORKLOAD["folding"], WORKLOAD["rate"], WORKLOAD["initial_reduction"],
              WORKLOAD["soundness_id"], WORKLOAD["security_level"])
    poly = O.rand_fe(WORKLOAD["seed"], 1 << k)
    groups = [[0]] * WORKLOAD["claims"]
    O.set_packed(True)  # Merkle hashing lane-packed, as the reference's packed Poseidon2
    for _ in range(args.warmup):
        O.prove(params, [poly], [k], groups)
    lat = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t = time.perf_counter()
        O.prove(params, [poly], [k], groups)
        lat.append(time.perf_counter() - t)
    el = time.perf_counter() - t0
    v = args.steps / el
    cores = O.lib().wo_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded Poly::rand)", "config": workload_config(k),
        "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)),
                       "p99": 1e3 * float(np.percentile(lat, 99))},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step one full proof of the 2^{k} workload "
                                   f"(oracle/ C restatement, Merkle hashing lane-packed as the "
                                   f"reference's packed Poseidon2; the Rust reference cannot be "
                                   f"built here: no cargo/rustc, Plonky3 not vendored)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _pct(v, q):
    return 1e3 * float(np.percentile(v, q)) if len(v) else None


def kernel_ms(W, ctx, fn):
    """GPU time of the library's kernels (DFT, leaf hash, tree, sumcheck
    classes, CUDA events on the context's stream) while fn() runs on ctx."""
    for klass in range(5):
        ctx.prof_read(klass)
    ctx.prof_enable_classes((W.PROF_DFT, W.PROF_LEAF, W.PROF_TREE, W.PROF_SUMCHECK))
    fn()
    ctx.prof_enable(False)
    return sum(ctx.prof_read(klass)[0] for klass in range(4))


def run_batched_verify(W, device, params, jobs):
    import concurrent.futures as cf
    proofs = [j.proof for j in jobs]
    want = [(0, j.checkpoint) for j in jobs]
    groups = [[0]] * 2
    vctx = W.Context(device)
    try:
        got = W.verify_batch(vctx, params, [16], groups, proofs)
        times = []
        for _ in range(5):
            t0 = time.perf_counter()
            W.verify_batch(vctx, params, [16], groups, proofs)
            times.append(time.perf_counter() - t0)
    finally:
        vctx.close()
    sub = proofs[:32]
    t0 = time.perf_counter()
    alone = [W.verify(params, [16], groups, p) for p in sub]
    t_one = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda p: W.verify(params, [16], groups, p), proofs[:threads]))
        t0 = time.perf_counter()
        pooled = list(ex.map(lambda p: W.verify(params, [16], groups, p), proofs))
        t_pool = time.perf_counter() - t0
    best = min(times)
    return {"workload": "the 256 proofs of batched_small verified (k=16, rate 1/4, folding 4, "
                        "2 claims)",
            "proofs_per_s": len(proofs) / best, "ms_per_batch": best * 1e3,
            "host_one_core_proofs_per_s": len(sub) / t_one,
            f"host_{threads}_threads_proofs_per_s": len(proofs) / t_pool,
            "speedup_vs_host_threads": (len(proofs) / best) / (len(proofs) / t_pool),
            "same_as_whir_verify": got == want and alone == want[:32] and pooled == want}


def run_batched(W, args, device):
    """Batched and served proving through the persistent worker pool
    (whir_server_*), each against the plain one-worker loop on the same jobs.

    The pool proves same-shape jobs that are queued together in lock step
    (one launch per pass for the whole group, whir_server_set_lockstep); the
    plain loop proves every job alone on one worker.

    batched_commit: 64 commitments, k uniform over 14..22 (log-uniform sizes),
    rate 1/2, folding 4; committed elements/s.  batched: 256 proofs at k=16 and
    16 at k=22, rate 1/4, folding 4, 2 claims each; proofs/s and completion
    p50/p99, beside the GPU-time cap: the 16 k=22 proofs cannot take less than
    16 times one k=22 proof's kernel time (their kernels fill the GPU), so the
    mix cannot exceed 272 proofs in that time.  served: Poisson arrivals at
    200, 400, 800 and 1600 req/s (--serve-jobs each), k uniform over 14..24, rate
    1/2 or 1/4, 1-4 claims, 150 GB device budget; sustained proofs/s and
    p50/p99 latency from arrival.  Inputs sit in pinned host memory; every
    proof of the pool is compared with the plain loop's proof of the same job.
    """
    import torch
    workers = args.workers or max(2, min(16, os.cpu_count() or 4))
    rng = np.random.default_rng(WORKLOAD["seed"] + 17)
    pool = {}
    for k in range(14, 25):
        t = torch.empty(1 << k, dtype=torch.int32, pin_memory=True)
        a = t.numpy().view(np.uint32)
        W.random_field(WORKLOAD["seed"] + 100 + k, 1 << k, out=a)
        pool[k] = (t, a)

    def params_of(k, rate):
        return (k, WORKLOAD["folding"], rate, WORKLOAD["initial_reduction"],
                WORKLOAD["soundness_id"], WORKLOAD["security_level"])

    def job(k, rate, claims, commit_only=False, arrival=0.0):
        return W.Job(params_of(k, rate), pool[k][1], claims=claims, commit_only=commit_only,
                     arrival_s=arrival)

    def same(a, b):
        return all(x.status == 0 and y.status == 0 and x.proof == y.proof and
                   x.checkpoint == y.checkpoint for x, y in zip(a, b))

    budget = 150 << 30
    srv = W.Server(workers=workers, device=device, budget_bytes=budget)
    one = W.Server(workers=1, device=device, budget_bytes=budget, lockstep=1)
    out = {"workers": workers, "lockstep_max_group": 64}
    try:
        # warm both pools up to the largest shape (buffers are kept)
        warm = [job(24, 2, 1) for _ in range(workers)]
        srv.run(warm)
        one.run([job(24, 2, 1)])

        # cfg: batched commitment
        ks = [int(x) for x in rng.integers(14, 23, 64)]
        mk = lambda: [job(k, 1, 0, commit_only=True) for k in ks]
        a, b = mk(), mk()
        srv.run(a)
        sa = min(srv.run(a)[0] for _ in range(3))
        one.run(b)
        sb, _ = one.run(b)
        elems = float(sum(1 << k for k in ks))
        out["batched_commit"] = {
            "workload": "64 commitments, k uniform over 14..22 (seeded), rate 1/2, folding 4",
            "elements_per_s": elems / sa, "plain_loop_elements_per_s": elems / sb,
            "speedup": sb / sa, "seconds": sa, "bit_exact_vs_plain": same(a, b)}

        # cfg: batched full proofs
        shapes = [16] * 256 + [22] * 16
        order = rng.permutation(len(shapes))
        mk = lambda: [job(shapes[i], 2, 2) for i in order]
        a, b = mk(), mk()
        srv.run(a)
        best = None
        for _ in range(3):
            a = mk()
            sa, peak = srv.run(a)
            if best is None or sa < best[0]:
                best = (sa, peak, a)
        sa, peak, a = best
        one.run(b)
        sb, _ = one.run(b)
        lat = [j.done_s for j in a]
        # GPU-time cap: one k=22 proof's kernel time, alone on a context
        cctx = W.Context(device)
        try:
            p22 = params_of(22, 2)
            W.prove_harness(cctx, p22, [pool[22][1]], [22], [[0]] * 2)
            t22 = min(kernel_ms(W, cctx, lambda: W.prove_harness(cctx, p22, [pool[22][1]], [22],
                                                                  [[0]] * 2)) for _ in range(3))
            p16 = params_of(16, 2)
            W.prove_batch(cctx, p16, [pool[16][1]] * 256, claims=2)
            t16 = kernel_ms(W, cctx, lambda: W.prove_batch(cctx, p16, [pool[16][1]] * 256,
                                                           claims=2))
        finally:
            cctx.close()
        cap = len(a) / (16 * t22 * 1e-3)
        out["batched"] = {
            "workload": "256 proofs at k=16 + 16 at k=22, rate 1/4, folding 4, 2 claims each",
            "proofs_per_s": len(a) / sa, "plain_loop_proofs_per_s": len(b) / sb,
            "speedup": sb / sa, "p50_ms": _pct(lat, 50), "p99_ms": _pct(lat, 99),
            "gpu_time_cap": {
                "proofs_per_s": cap, "frac": (len(a) / sa) / cap,
                "speedup_vs_plain_at_cap": cap / (len(b) / sb),
                "k22_proof_kernel_ms": t22, "k16_proof_kernel_ms_in_group_of_256": t16 / 256,
                "note": "272 proofs in 16 x the kernel time of one k=22 proof alone"},
            "peak_device_gb": peak / 2 ** 30, "bit_exact_vs_plain": same(a, b)}

        # the small proofs of the mix alone: 256 at k=16
        mk = lambda: [job(16, 2, 2) for _ in range(256)]
        a, b = mk(), mk()
        srv.run(a)
        sa = min(srv.run(mk())[0] for _ in range(3))
        a = mk()
        srv.run(a)
        one.run(b)
        sb, _ = one.run(b)
        out["batched_small"] = {
            "workload": "256 proofs at k=16, rate 1/4, folding 4, 2 claims each",
            "proofs_per_s": len(a) / sa, "plain_loop_proofs_per_s": len(b) / sb,
            "speedup": sb / sa, "bit_exact_vs_plain": same(a, b)}

        # those 256 proofs verified: whir_verify_batch (transcript passes on
        # host threads, every Merkle opening of every proof in one launch)
        # against whir_verify one proof at a time, on one core and on a
        # thread per host core
        out["batched_verify"] = run_batched_verify(W, device, params_of(16, 2), a)

        # cfg: served Poisson stream, an arrival-rate sweep
        sweep = []
        for lam in (200, 400, 800, 1600):
            arr, t = [], 0.0
            for _ in range(args.serve_jobs):
                t += float(rng.exponential(1 / lam))
                arr.append(t)
            spec = [(int(rng.integers(14, 25)), int(rng.choice([1, 2])), int(rng.integers(1, 5)))
                    for _ in arr]
            mk = lambda: [job(kk, r, c, arrival=x) for (kk, r, c), x in zip(spec, arr)]
            a, b = mk(), mk()
            sa, peak = srv.run(a, serve=True)
            sb, _ = one.run(b, serve=True)
            la = [j.latency_s for j in a]
            lb = [j.latency_s for j in b]
            sweep.append({
                "arrivals_per_s": lam, "jobs": len(a),
                "proofs_per_s": len(a) / sa, "p50_ms": _pct(la, 50), "p99_ms": _pct(la, 99),
                "serial_plain": {"proofs_per_s": len(b) / sb, "p50_ms": _pct(lb, 50),
                                 "p99_ms": _pct(lb, 99)},
                "throughput_ratio": sb / sa,
                "peak_device_gb": peak / 2 ** 30, "bit_exact_vs_plain": same(a, b)})
        # GPU time of the saturated stream's jobs, each proved alone: the
        # summed single-proof kernel time of the 400 jobs (lock-step groups
        # can beat it for the small shapes; the large ones fill the GPU alone)
        kt = {}
        kctx = W.Context(device)
        try:
            for (kk, r, c) in sorted(set(spec)):
                pk = params_of(kk, r)
                W.prove_harness(kctx, pk, [pool[kk][1]], [kk], [[0]] * c)
                kt[(kk, r, c)] = kernel_ms(W, kctx, lambda: W.prove_harness(
                    kctx, pk, [pool[kk][1]], [kk], [[0]] * c))
        finally:
            kctx.close()
        gpu_s = sum(kt[x] for x in spec) * 1e-3
        sweep[-1]["gpu_time_of_jobs_alone"] = {
            "proofs_per_s": len(spec) / gpu_s,
            "frac": sweep[-1]["proofs_per_s"] / (len(spec) / gpu_s),
            "note": "jobs / summed kernel time of each job proved alone"}
        # the knee: the lowest rate at which the serial loop no longer keeps up
        knee = next((s["arrivals_per_s"] for s in sweep
                     if s["serial_plain"]["proofs_per_s"] < 0.9 * s["arrivals_per_s"]), None)
        top = sweep[-1]
        out["served"] = {
            "workload": f"Poisson arrivals, {args.serve_jobs} jobs per rate, k uniform over "
                        "14..24, rate 1/2 or 1/4, folding 4, 1-4 claims, 150 GB budget",
            "sweep": sweep, "serial_plain_knee_arrivals_per_s": knee,
            "saturated": {"arrivals_per_s": top["arrivals_per_s"],
                          "proofs_per_s": top["proofs_per_s"],
                          "serial_plain_proofs_per_s": top["serial_plain"]["proofs_per_s"],
                          "throughput_ratio": top["throughput_ratio"],
                          "gpu_time_of_jobs_alone": top["gpu_time_of_jobs_alone"]},
            "bit_exact_vs_plain": all(s["bit_exact_vs_plain"] for s in sweep)}
    finally:
        srv.close()
        one.close()
    return out


# The reference's own benchmark test, whir_bench (crates/whir/src/test.rs:284-290):
# k = 25, folding 5, rate 1/2, initial_reduction 3, JohnsonBound, 123-bit, 1 claim.
WHIR_BENCH_SHAPE = dict(k=25, folding=5, rate=1, initial_reduction=3, soundness_id=1,
                        security_level=123, claims=1, seed=1)


def run_whir_bench_shape(W, ctx, stream, steps=10, warmup=3):
    """Plain proofs at whir_bench's shape, polynomial resident in HBM, timed
    with CUDA events on the prover's stream (a secondary line: the headline
    workload is the k = 24 one)."""
    import torch
    s = WHIR_BENCH_SHAPE
    k = s["k"]
    params = (k, s["folding"], s["rate"], s["initial_reduction"], s["soundness_id"],
              s["security_level"])
    whir = W.Whir(ctx, *params)
    dev = ctx.to_device(W.random_field(s["seed"], 1 << k))
    groups = [[0]] * s["claims"]

    def one():
        t = W.PoseidonWriter()
        whir.prove(t, dev, [k], groups)
        t.draw_base()
        return t

    for _ in range(warmup):
        proof = one().finalize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    evs[0].record(stream)
    for i in range(steps):
        one()
        evs[i + 1].record(stream)
    evs[-1].synchronize()
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    whir.close()
    dev.close()
    return {"config": {"workload": "whir_bench shape: k=25 (2^25 KoalaBear), rate 1/2, folding 5, "
                                   "initial_reduction 3, JohnsonBound, 123-bit, 1 claim",
                       "polynomial": "resident in HBM"},
            "proofs_per_s": steps / (total_ms * 1e-3), "ms_per_proof": total_ms / steps,
            "latency_ms": {"p50": float(np.percentile(lat, 50)),
                           "p99": float(np.percentile(lat, 99))},
            "proof_bytes": len(proof), "steps": steps, "warmup": warmup}, proof


def cpu_whir_bench_shape(expect_proof):
    """One oracle proof at whir_bench's shape on the host cores, compared with
    the GPU's proof bytes."""
    from oracle import oracle as O
    s = WHIR_BENCH_SHAPE
    k = s["k"]
    params = (k, s["folding"], s["rate"], s["initial_reduction"], s["soundness_id"],
              s["security_level"])
    poly = O.rand_fe(s["seed"], 1 << k)
    O.set_packed(True)
    try:
        t0 = time.perf_counter()
        proof, _ = O.prove(params, [poly], [k], [[0]] * s["claims"])
        el = time.perf_counter() - t0
    finally:
        O.set_packed(False)
    return {"value": 1.0 / el, "unit": UNIT, "cores": O.lib().wo_threads(), "kind": "port",
            "sample": f"1 full proof in {el:.1f} s (oracle/: C restatement, OpenMP, lane-packed "
                      f"Merkle hashing)",
            "gpu_proof_identical": bool(proof == expect_proof)}


# The reference's Merkle benchmarks (crates/merkle/src/lib.rs:314-349, 384-420):
# commit and one query of 2^21 rows of 32 base elements, and of 2^18 rows of 32
# extension elements (128 words).
MERKLE_BENCH_SHAPES = [("bench_merkle_base_packed", 21, 32), ("bench_merkle_ext_packed", 18, 128)]


def run_merkle_bench_shapes(W, ctx, steps=10, warmup=3):
    """Commit + one opening through the public ABI (whir_merkle_commit, which
    reserves the tree, hashes the rows, builds the levels and reads the root
    back, then whir_merkle_open), rows resident in HBM, host clock per call."""
    out = {}
    for name, k, row_len in MERKLE_BENCH_SHAPES:
        rows = ctx.to_device(W.random_field(0, row_len << k))

        def one():
            t = W.MerkleTree(ctx, rows, k, row_len)
            t.open([(5 << k) // 7])
            t.close()

        for _ in range(warmup):
            one()
        lat = []
        for _ in range(steps):
            t0 = time.perf_counter()
            one()
            lat.append(time.perf_counter() - t0)
        rows.close()
        ms = 1e3 * float(np.mean(lat))
        perm24 = (row_len // 16) << k
        perm16 = (1 << k) - 1
        out[name] = {"rows": 1 << k, "row_words": row_len, "ms_per_commit_and_query": ms,
                     "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                     "leaf_perm24_per_s": perm24 / (ms * 1e-3),
                     "tree_perm16": perm16, "steps": steps, "warmup": warmup}
    return out


def run_gb300(args):
    import torch
    import whir_gb300 as W

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    k = args.k
    ctx = W.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    params = (k, WORKLOAD["folding"], WORKLOAD["rate"], WORKLOAD["initial_reduction"],
              WORKLOAD["soundness_id"], WORKLOAD["security_level"])
    whir = W.Whir(ctx, *params)
    poly = W.random_field(WORKLOAD["seed"], 1 << k)
    groups = [[0]] * WORKLOAD["claims"]
    dev_poly = ctx.to_device(poly)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def prove_dev():
        t = W.PoseidonWriter()
        whir.prove(t, dev_poly, [k], groups)
        t.draw_base()
        return t

    # launch splits of this device for the workload's tree heights and DFT
    # sizes (untimed; outputs do not depend on them)
    tune_report = "" if args.no_autotune else W.autotune(
        ctx, 10, k + WORKLOAD["rate"] - WORKLOAD["folding"])
    for _ in range(args.warmup):
        first = prove_dev()
    gpu_proof = first.finalize()

    # ---- value: device-resident input ----
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize(local)
    for klass in range(5):
        ctx.prof_read(klass)
    # events around the leaf-hash launches (the dominant kernel, five per
    # proof) and host clocks around the waits; the other classes are timed
    # in a second pass below (events on every launch cost about 1% of the
    # proof time)
    ctx.prof_enable_classes((W.PROF_LEAF, W.PROF_SYNC))
    launches0, _, _ = ctx.counters()
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    wall0 = time.perf_counter()
    for i in range(args.steps):
        prove_dev()
        evs[i + 1].record(stream)
    evs[-1].synchronize()
    wall_ms = 1e3 * (time.perf_counter() - wall0)
    clk = clocks.stop()
    launches1, _, _ = ctx.counters()
    ctx.prof_enable(False)
    barrier()
    total_ms = evs[0].elapsed_time(evs[-1])
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    prof = {}

    def class_stats(klass, steps, note=None):
        ms, n, b = ctx.prof_read(klass)
        d = {"ms_per_step": ms / steps, "launches_per_step": n / steps,
             "share": ms / steps / (total_ms / args.steps) if total_ms else None,
             "achieved_gbs": (b / (ms * 1e-3) / 1e9) if ms else None,
             "bytes_per_step": b / steps}
        if note:
            d["note"] = note
        return d

    prof["leaf_hash"] = class_stats(1, args.steps)
    sync_ms, sync_n, _ = ctx.prof_read(4)
    # DFT, tree and sumcheck passes: a shorter pass with their events on
    sc_steps = max(3, args.steps // 3)
    ctx.prof_enable_classes((W.PROF_DFT, W.PROF_TREE, W.PROF_SUMCHECK))
    for _ in range(sc_steps):
        prove_dev()
    torch.cuda.synchronize(local)
    ctx.prof_enable(False)
    note = f"timed in a separate pass of {sc_steps} proofs"
    prof["dft"] = class_stats(0, sc_steps, note)
    prof["merkle_tree"] = class_stats(2, sc_steps, note)
    prof["sumcheck"] = class_stats(3, sc_steps, note)
    prof["host_wait"] = {"ms_per_step": sync_ms / args.steps, "waits_per_step": sync_n / args.steps,
                         "share": sync_ms / total_ms if total_ms else None,
                         "note": "host time blocked on the stream (transcript round trips)"}
    prof["wall_ms_per_step"] = wall_ms / args.steps
    total_ms = max_over_ranks(total_ms, world, f"cuda:{local}")
    value = replica_throughput(world, args.steps, total_ms * 1e-3)

    # ---- e2e: pinned host input through the C ABI ----
    host_t = torch.empty(1 << k, dtype=torch.int32, pin_memory=True)
    host = host_t.numpy().view(np.uint32)
    host[:] = poly

    def prove_host():
        t = W.PoseidonWriter()
        whir.prove(t, host, [k], groups)
        t.draw_base()
        return t.finalize()

    prove_host()
    barrier()
    torch.cuda.synchronize(local)
    _, h2d0, d2h0 = ctx.counters()
    t0 = time.perf_counter()
    e2e_lat = []
    for i in range(args.steps):
        ts = time.perf_counter()
        prove_host()
        e2e_lat.append(time.perf_counter() - ts)
    e2e_s = time.perf_counter() - t0
    _, h2d1, d2h1 = ctx.counters()
    barrier()
    e2e_s = max_over_ranks(e2e_s, world, f"cuda:{local}")

    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    kern = {n: v for n, v in prof.items() if n in ("dft", "leaf_hash", "merkle_tree", "sumcheck")}
    dom = max(kern, key=lambda n: kern[n]["ms_per_step"])
    d = prof[dom]
    per_launch_ms = d["ms_per_step"] / max(d["launches_per_step"], 1e-9)
    achieved = d["achieved_gbs"]
    traffic = NCU_TRAFFIC_BYTES.get(dom) if k == NCU_TRAFFIC_K else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded Poly::rand, as the reference harness)",
        "config": workload_config(k),
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "e2e": {"value": replica_throughput(world, args.steps, e2e_s), "unit": UNIT,
                "h2d_bytes_per_step": (h2d1 - h2d0) / args.steps,
                "d2h_bytes_per_step": (d2h1 - d2h0) / args.steps,
                "latency_ms": {"p50": 1e3 * float(np.percentile(e2e_lat, 50)),
                               "p99": 1e3 * float(np.percentile(e2e_lat, 99))}},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak if achieved else None,
                     "peak_source": peak_src, "traffic": traffic,
                     "per_launch_ms": per_launch_ms,
                     "limiter": "integer pipes, not HBM: see integer_pipe (frac of the issue "
                                "bound); this HBM frac only shows the memory side is idle"},
        "integer_pipe": integer_roofline(k, prof, clk),
        "kernels": prof,
        "gpu_launches": int(launches1 - launches0),
        "autotune": tune_report.splitlines(),
        "clocks": clk,
    }
    if not args.no_batched:
        line["batched_served"] = run_batched(W, args, local)
    if not args.no_whir_bench_shape:
        line["whir_bench_shape"], wb_proof = run_whir_bench_shape(W, ctx, stream)
        line["merkle_bench_shapes"] = run_merkle_bench_shapes(W, ctx)
        if not args.no_cpu_baseline and world == 1:
            line["whir_bench_shape"]["cpu_baseline"] = cpu_whir_bench_shape(wb_proof)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(k, args.cpu_seconds, expect_proof=gpu_proof)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
