"""Benchmark: wavelet-tree + rank/select build throughput on GB300.

Workload (one step): a full build of the integer wavelet tree over
n = 2^30 uint32 symbols drawn as min(floor(Exp(mean 2^14)), 2^20 - 1)
(seeded), 20 levels (sigma 2^20, wt_int max_level semantics), with
rank_support_v<1>, select_support_mcl<1> and select_support_mcl<0> over the
concatenated 20 x 2^30-bit level bitvector.

  value : algorithmic GB/s of the whole build with the input resident in HBM
  e2e   : the same through the host API from pinned host memory:
          wtg_tree_build_out (input copied in, bits and rank table copied
          back while the build runs) plus the select tables' getters
The algorithmic bytes of one build are
  L*n*w (level reads) + (L-1)*n*w (next-level writes) + L*n/8 (bits)
  + [L*n/8 + 16*((L*n>>9)+1)] (rank: read bits, write table)
  + 2 * [L*n/8 + select sample bytes written] (select1, select0).

--impl reference times the reference's own CPU code on the host cores instead:
levelWT's WT() (-DLONG -DINT, OpenMP) and rank_support_v_par +
select_support_mcl_par<1>/<0> (OpenMP), built from the reference's sources by
oracle/Makefile (bench-ref), on a bounded sample of the workload per step; where
those builds are absent it times the oracle's restatement of the same code
("kind": "port").

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl wtg|reference]
Multi-GPU (torchrun): every rank builds its own independent sequence; no
collective touches the data path (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "wavelet-suffix-fm-index_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "WT+rank/select build GB/s (% HBM peak); select Mq/s learned vs plain, exact"
WORKLOAD = "wt_int build, n=2^30 uint32, Exp(mean 2^14) clamped to 2^20-1, 20 levels, rank + select1 + select0"
MEAN, CAP, LEVELS, SEED = 2 ** 14, 2 ** 20 - 1, 20, 20240611


def algorithmic_bytes(n, L, w, sel_words=0):
    nb = n * L
    bits = nb / 8
    return (L * n * w + (L - 1) * n * w + bits + (bits + 16 * ((nb >> 9) + 1)) + 2 * bits + 8 * sel_words)


# DRAM bytes (read + write) per symbol of one uint32 partitioning level pass,
# from ncu's dram__bytes_read.sum + dram__bytes_write.sum over three level
# launches (levels 9-11) of an n=2^28 build: 2137.7 MB per launch (1079.0 MB
# read, 1058.7 MB written) against 2181.0 MB algorithmic; traffic grows
# linearly with n, so a full launch's traffic is this figure times n.
LEVEL_DRAM_BYTES_PER_SYMBOL_U32 = 2137.7e6 / 2 ** 28


def level_launch_bytes(n, w):
    """Algorithmic bytes of one partitioning level pass: read n symbols,
    write n symbols, write n bits."""
    return 2 * n * w + n / 8


def init_ranks(dist, backend, timeout_s):
    """The process group of a multi-rank run, with a short timeout: a rank
    that fails or leaves between steps ends the others' next collective with
    an error instead of a hang."""
    import datetime
    dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))


def slowest_rank(dist, torch, seconds, device):
    """The job's time: the maximum of one value over all ranks (identity
    without a process group)."""
    if not dist:
        return seconds
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, steps, step_bytes, seconds):
    """Whole-job GB/s: every rank builds its own sequence of step_bytes per
    step (replicas), all finishing within `seconds` (the slowest rank)."""
    return world * steps * step_bytes / seconds / 1e9


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload_config(n, world):
    """The `config` of both arms' lines (the workload, not the sample)."""
    return {"workload": WORKLOAD, "n": n, "levels": LEVELS, "sigma": 1 << LEVELS, "elem_bytes": 4,
            "l2": "inputs larger than L2 (4 GiB per level pass, 2.5 GiB of bits)",
            "parallelism": f"replicas x{world} (independent sequences)"}


def cpu_reference_seconds(n):
    """One build of an n-symbol sample of the workload by the reference's own
    code (levelWT WT() with -DLONG -DINT, then rank_support_v_par and
    select_support_mcl_par<1>/<0> over its bits, all OpenMP threads).
    Returns (seconds, algorithmic bytes, cores), or None where the
    reference's builders are not built."""
    import datagen
    from oracle import oracle as O
    if O.ref_bench() is None:
        return None
    sym = datagen.exp_u32(n, mean=MEAN, cap=CAP, seed=SEED)
    t_wt, t_r, t_s1, t_s0, sel_words = O.ref_bench_times(sym, LEVELS)
    return t_wt + t_r + t_s1 + t_s0, algorithmic_bytes(n, LEVELS, 4, sel_words), O.num_threads()


def cpu_build_seconds(n, threads_note=True):
    """One full CPU build (oracle restatement, all OpenMP threads) of an n-symbol
    sample of the workload; returns (seconds, sample bytes, cores)."""
    import datagen
    from oracle import oracle as O
    sym = datagen.exp_u32(n, mean=MEAN, cap=CAP, seed=SEED)
    t0 = time.perf_counter()
    bits, _ = O.wt_build(sym, LEVELS)
    w = np.concatenate([bits, np.zeros(1, np.uint64)])
    O.rank_build(w, n * LEVELS)
    s1 = O.Select(w, n * LEVELS, 1)
    s0 = O.Select(w, n * LEVELS, 0)
    dt = time.perf_counter() - t0
    sel_words = s1.sb_nwords + s1.nsb + s1.pool_nwords + s0.sb_nwords + s0.nsb + s0.pool_nwords
    return dt, algorithmic_bytes(n, LEVELS, 4, sel_words), O.num_threads()


def run_reference(args, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(ref=True)
    n = 1 << args.cpu_log2
    kind = "reference" if O.ref_bench() is not None else "port"
    timed = cpu_reference_seconds if kind == "reference" else cpu_build_seconds
    for _ in range(args.warmup):
        timed(n)
    tot_t, tot_b, cores = 0.0, 0.0, 1
    for _ in range(args.steps):
        dt, b, cores = timed(n)
        tot_t += dt
        tot_b += b
    gbs = tot_b / tot_t / 1e9
    what = ("the reference's levelWT WT() (-DLONG -DINT) + rank_support_v_par + select_support_mcl_par<1>/<0>, "
            "OpenMP" if kind == "reference" else "the oracle's restatement of levelWT + rank/select, OpenMP")
    sample = f"n=2^{args.cpu_log2} uint32 symbols of the same distribution, 20 levels, one full build per step: {what}"
    line = {
        "impl": "reference", "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(1 << args.n_log2, 1),
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def select_queries(torch, m_levels, nq, gen, dev):
    """nq uniform-random (level, k) select queries: the level uniform over the
    levels holding at least one arg, k uniform in [1, args of the level]."""
    valid = [l for l, m in enumerate(m_levels) if m > 0]
    vl = torch.tensor(valid, device=dev, dtype=torch.int64)
    mt = torch.tensor([m_levels[l] for l in valid], device=dev, dtype=torch.float64)
    idx = torch.randint(0, len(valid), (nq,), device=dev, generator=gen)
    k = torch.floor(torch.rand(nq, device=dev, dtype=torch.float64, generator=gen) * mt[idx]).to(torch.int64) + 1
    k = torch.minimum(k, mt[idx].to(torch.int64))
    return vl[idx].contiguous(), k.contiguous()


def measure_queries(torch, tree, seq, n, dev, stream, log2_q, reps=5):
    """wt_int access, rank(i, c), lex_count(i, j, c) and range_search_2d
    counts: 2^log2_q queries each; positions uniform, i uniform in [0, n], c
    drawn from the input, j - i and rb - lb uniform below 2^20, value window
    [c - 2^12, c + 2^12]."""
    sp = stream.cuda_stream
    nq = 1 << log2_q
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + 11)
    idx = torch.randint(0, n, (nq,), device=dev, generator=gen, dtype=torch.int64)
    ri = torch.randint(0, n + 1, (nq,), device=dev, generator=gen, dtype=torch.int64)
    rc = seq[torch.randint(0, n, (nq,), device=dev, generator=gen, dtype=torch.int64)].to(torch.int64)
    out = torch.empty(nq, device=dev, dtype=torch.int64)
    # range queries: [i, j) of up to 2^20 positions; value window c +- 2^12
    span = torch.randint(0, 1 << 20, (nq,), device=dev, generator=gen, dtype=torch.int64)
    rj = torch.clamp(ri + span, max=n)
    rb = torch.clamp(idx + span, max=n - 1)
    vlb = torch.clamp(rc - (1 << 12), min=0)
    vrb = rc + (1 << 12)
    o2 = torch.empty(nq, device=dev, dtype=torch.int64)
    o3 = torch.empty(nq, device=dev, dtype=torch.int64)
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    res = {}
    for name, fn in (("access", lambda: tree.access_device(idx.data_ptr(), nq, out.data_ptr(), sp)),
                     ("rank", lambda: tree.rank_device(ri.data_ptr(), rc.data_ptr(), nq, out.data_ptr(), sp)),
                     ("lex_count", lambda: tree.lex_count_device(ri.data_ptr(), rj.data_ptr(), rc.data_ptr(), nq,
                                                                 out.data_ptr(), o2.data_ptr(), o3.data_ptr(), sp)),
                     ("range_count", lambda: tree.range_count_device(idx.data_ptr(), rb.data_ptr(), vlb.data_ptr(),
                                                                     vrb.data_ptr(), nq, out.data_ptr(), sp))):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[name] = {"mqs": nq / (ms / 1e3) / 1e6, "ms": ms}
    # access must give back the input
    tree.access_device(idx.data_ptr(), nq, out.data_ptr(), sp)
    torch.cuda.synchronize()
    res["access_exact"] = bool(torch.equal(out, seq[idx].to(torch.int64)))
    # a full value window counts every position of [lb, rb]
    zero = torch.zeros_like(idx)
    top = torch.full_like(idx, 1 << tree.levels)
    tree.range_count_device(idx.data_ptr(), rb.data_ptr(), zero.data_ptr(), top.data_ptr(), nq, out.data_ptr(), sp)
    torch.cuda.synchronize()
    res["range_exact"] = bool(torch.equal(out, rb - idx + 1))
    res["queries"] = nq
    return res


def measure_fm(torch, wtg, oracle_mod, dev, log2_n, log2_q, cpu_log2):
    """FM-index core on an order-2 Markov DNA text of 2^log2_n symbols with
    0.1 % N runs and a '$' terminator: suffix array + BWT
    (fm-index/par/WT.C:33-41) on the GPU,
    the 3-level wavelet tree of the BWT codes with rank + select, and 2^log2_q
    backward-search counts of patterns of U[8, 32] symbols copied from the
    text (each occurs, so every count must be >= 1: counts_below_1 = 0).  The CPU figure is the
    oracle's suffix array on a 2^cpu_log2 sample (single thread)."""
    import datagen
    n = 1 << log2_n
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    with torch.cuda.stream(stream):
        text = datagen.dna_markov_device(n, torch, dev, seed=SEED + 17)
        # a unique smallest last symbol: suffix order is then rotation order,
        # so backward search over the sentinel-free BWT counts exactly
        text[n - 1] = ord("$")
        sa = torch.empty(n, dtype=torch.int32, device=dev)
        bw = torch.empty(n, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    rounds = wtg.suffix_array_device(text.data_ptr(), n, sa.data_ptr(), bw.data_ptr(), sp)  # warm-up
    reps = 2
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(reps):
        wtg.suffix_array_device(text.data_ptr(), n, sa.data_ptr(), bw.data_ptr(), sp)
    e1.record(stream)
    torch.cuda.synchronize()
    sa_ms = e0.elapsed_time(e1) / reps
    # BWT bytes -> codes 0..sigma-1 in byte order, then its wavelet tree
    with torch.cuda.stream(stream):
        present = torch.zeros(256, dtype=torch.int64, device=dev)
        present[torch.unique(bw).long()] = 1
        lut = (torch.cumsum(present, 0) - 1).to(torch.uint8)
        codes = lut[bw.long()].contiguous()
        tcodes = lut[text.long()].contiguous()
    torch.cuda.synchronize()
    sigma = int(present.sum().item())
    fm = wtg.FMIndex.from_device(codes.data_ptr(), n, sigma, sp)
    e0, e1 = ev(), ev()
    e0.record(stream)
    fm2 = wtg.FMIndex.from_device(codes.data_ptr(), n, sigma, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    wt_ms = e0.elapsed_time(e1)
    del fm2
    # count queries
    nq = 1 << log2_q
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 19)
    lens = torch.randint(8, 33, (nq,), device=dev, generator=g)
    starts = torch.randint(0, n - 32, (nq,), device=dev, generator=g)
    off = torch.zeros(nq + 1, dtype=torch.int64, device=dev)
    off[1:] = torch.cumsum(lens, 0)
    total = int(off[-1].item())
    qid = torch.repeat_interleave(torch.arange(nq, device=dev), lens)
    pos = starts[qid] + (torch.arange(total, device=dev) - off[:-1][qid])
    pat = tcodes[pos].contiguous()
    patb = text[pos].contiguous()  # the same patterns as bytes, for the Huffman-shaped tree
    del qid, pos
    dC = torch.from_numpy(fm.C.view(np.int64)).to(dev)
    out = torch.empty(nq, dtype=torch.int64, device=dev)
    run = lambda: fm.count_device(dC.data_ptr(), pat.data_ptr(), off.data_ptr(), nq, out.data_ptr(), sp)  # noqa: E731
    run()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(3):
        run()
    e1.record(stream)
    torch.cuda.synchronize()
    q_ms = e0.elapsed_time(e1) / 3
    zero = int((out < 1).sum().item())
    # the reference FM-index's own tree (fm-index/par/WT.C:44): wt_huff over
    # the BWT's bytes; the same patterns must give the same counts
    hf = wtg.HuffmanTree.from_device(bw.data_ptr(), n, wtg.ALL, sp)
    hf.free()
    e0, e1 = ev(), ev()
    e0.record(stream)
    hf = wtg.HuffmanTree.from_device(bw.data_ptr(), n, wtg.ALL, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    huff_ms = e0.elapsed_time(e1)
    hist = torch.bincount(text.long(), minlength=256)
    dCb = torch.zeros(256, dtype=torch.int64, device=dev)
    dCb[1:] = torch.cumsum(hist, 0)[:-1]
    outh = torch.empty(nq, dtype=torch.int64, device=dev)
    runh = lambda: hf.fm_count_device(dCb.data_ptr(), patb.data_ptr(), off.data_ptr(), nq, outh.data_ptr(), sp)  # noqa: E731
    runh()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(3):
        runh()
    e1.record(stream)
    torch.cuda.synchronize()
    hq_ms = e0.elapsed_time(e1) / 3
    huff = {"build_ms": huff_ms, "bits": hf.size, "nodes": hf.num_nodes, "count_ms": hq_ms,
            "count_mqs": nq / (hq_ms / 1e3) / 1e6, "counts_equal_balanced_tree": bool(torch.equal(out, outh))}
    hf.free()
    del patb, outh, dCb
    # sorted-order spot check of the suffix array: adjacent suffixes compare
    # by first symbol, then by the inverse array one position on
    s_h = text.cpu().numpy()
    sa_h = sa.cpu().numpy().astype(np.int64)
    inv = np.empty(n + 1, np.int64)
    inv[sa_h] = np.arange(n)
    inv[n] = -1
    a_, b_ = sa_h[:-1], sa_h[1:]
    sa_exact = bool(((s_h[a_] < s_h[b_]) | ((s_h[a_] == s_h[b_]) & (inv[a_ + 1] < inv[b_ + 1]))).all())
    del s_h, sa_h, inv, a_, b_
    cpu = None
    if oracle_mod is not None and cpu_log2:
        m = 1 << cpu_log2
        sample = text[:m].cpu().numpy()
        t0 = time.perf_counter()
        oracle_mod.suffix_array(sample)
        cpu_s = time.perf_counter() - t0
        cpu = {"symbols_per_s": m / cpu_s, "sample": f"first 2^{cpu_log2} symbols, oracle prefix doubling, 1 thread",
               "s": cpu_s}
    res = {"workload": f"order-2 Markov DNA text + '$', n=2^{log2_n}, 0.1% N runs; SA+BWT, 3-level WT + rank + select "
                       f"of the BWT, 2^{log2_q} counts of patterns of U[8,32] symbols",
           "n": n, "sigma": sigma, "sa_bwt_ms": sa_ms, "sa_rounds": rounds,
           "sa_msym_per_s": n / (sa_ms / 1e3) / 1e6, "wt_ms": wt_ms, "fm_build_ms": sa_ms + wt_ms,
           "count_queries": nq, "count_ms": q_ms, "count_mqs": nq / (q_ms / 1e3) / 1e6,
           "counts_below_1": zero, "sa_order_exact": sa_exact, "huff": huff, "cpu_suffix_array": cpu}
    del text, sa, bw, codes, tcodes, pat, fm
    torch.cuda.empty_cache()
    return res


def b_texts_host(texts_seed, ntexts):
    """The batch workload's texts on the host (the generator of measure_batch)."""
    rng = np.random.default_rng(texts_seed)
    lengths = np.floor(2.0 ** rng.uniform(10, 20, ntexts)).astype(np.uint64)
    concat = rng.integers(0, 4, int(lengths.sum()), dtype=np.uint8)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    return [concat[offs[t]:offs[t + 1]] for t in range(ntexts)]


def measure_batch(torch, wtg, stream, ntexts, reps=5, cpu_texts=0, shape=None):
    """Batched build of ntexts DNA-like texts (lengths floor(2^U[10,20]),
    i.i.d. uniform over 4 symbols, 2 levels, rank + select1 + select0): one
    persistent launch replayed from a CUDA graph, against the same texts
    built one by one through the single-sequence device API."""
    import ctypes
    rng = np.random.default_rng(SEED + 13)
    lengths = np.floor(2.0 ** rng.uniform(10, 20, ntexts)).astype(np.uint64)
    total = int(lengths.sum())
    texts = rng.integers(0, 4, total, dtype=np.uint8)
    stream = torch.cuda.Stream()  # the batch runs and is timed on its own stream
    b = wtg.Batch(lengths, 2, wtg.ALL, stream.cuda_stream)
    b.load(texts)
    del texts
    if shape:  # (split tile, whole-text bound, symbols per thread) instead of the tuner's choice
        b.set_shape(*shape)
    t0 = time.perf_counter()
    b.run()  # first run: autotune (unless the shape is fixed) + graph capture
    b.sync()
    first_s = time.perf_counter() - t0
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for _ in range(3):
        b.run()
    b.sync()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(reps):
        b.run()
    e1.record(stream)
    b.sync()
    ms = e0.elapsed_time(e1) / reps
    step_bytes = sum(algorithmic_bytes(int(n), 2, 1) for n in lengths)
    tile, whole_max, spt, nwhole, tune_ms = b.shape()
    # the same texts, one single-sequence build each
    d_in, _ = b.input_device()
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)
    L_ = wtg.lib()
    h = ctypes.c_void_p()
    sp = ctypes.c_void_p(stream.cuda_stream)
    wtg._ck(L_.wtg_tree_build_device(ctypes.c_void_p(d_in), int(lengths[0]), 1, 2, wtg.ALL, sp, ctypes.byref(h)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(ntexts):
        wtg._ck(L_.wtg_tree_build_device(ctypes.c_void_p(d_in + int(offs[t])), int(lengths[t]), 1, 2, wtg.ALL, sp,
                                         ctypes.byref(h)))
    wtg._ck(L_.wtg_tree_sync(h))
    plain_s = time.perf_counter() - t0
    L_.wtg_tree_free(h)
    # spot check: the batch's outputs for a few texts equal the single builds
    exact = True
    for t in rng.choice(ntexts, 4, replace=False):
        t = int(t)
        ref = wtg.WaveletTree.from_device(d_in + int(offs[t]), int(lengths[t]), 1, 2, wtg.ALL, stream.cuda_stream)
        ref.sync()
        exact = exact and np.array_equal(b.bits(t), ref.bits()) and \
            np.array_equal(b.rank_table(t), ref.rank_table()) and \
            np.array_equal(b.select_tables(t, 0).pool, ref.select_tables(0).pool)
        ref.free()
    b.free()
    cpu = None
    if cpu_texts:
        from oracle import oracle as O
        if O.ref_bench() is not None:
            # every (ntexts / cpu_texts)-th text: the reference's WT() per text
            # and its rank/select constructors per text, OpenMP across texts
            pick = np.arange(0, ntexts, max(1, ntexts // cpu_texts))
            h_texts = b_texts_host(texts_seed=SEED + 13, ntexts=ntexts)
            lens_s = lengths[pick]
            concat_s = np.concatenate([h_texts[int(t)] for t in pick])
            t_wt, t_rs = O.ref_bench_batch(concat_s, lens_s, 2)
            sb = sum(algorithmic_bytes(int(m), 2, 1) for m in lens_s)
            cpu = {"value": sb / (t_wt + t_rs) / 1e9, "unit": "GB/s", "cores": O.num_threads(), "kind": "reference",
                   "sample": f"{pick.size} of the {ntexts} texts ({int(lens_s.sum())} symbols): the reference's WT() "
                             "and rank_support_v + select_support_mcl<1>/<0> constructors per text, OpenMP across texts",
                   "wt_s": t_wt, "supports_s": t_rs}
    return {
        "workload": f"{ntexts} texts, lengths floor(2^U[10,20]), uniform over 4 symbols, 2 levels, "
                    "rank + select1 + select0 per text",
        "cpu_baseline": cpu,
        "texts": ntexts, "symbols": total, "algorithmic_bytes": step_bytes,
        "ms": ms, "gbs": step_bytes / (ms / 1e3) / 1e9, "first_run_s": first_s,
        "shape": {"split_tile_symbols": tile, "whole_text_max_symbols": whole_max, "symbols_per_thread": spt,
                  "texts_built_whole": nwhole, "candidates_ms": [round(float(x), 3) for x in tune_ms[:6]]},
        "per_text_plain_ms": plain_s * 1e3, "per_text_plain_gbs": step_bytes / plain_s / 1e9,
        "speedup_vs_per_text": plain_s * 1e3 / ms, "exact_spot_check": bool(exact),
    }


def measure_byte_text(torch, wtg, dev, log2_n, reps=10, cpu=True):
    """The byte-text build: n = 2^log2_n uint8 symbols, Zipf(1.0) over the 256
    byte values (seeded rank -> byte permutation), 8 levels (levelWT's tree
    for sigma 256), rank_support_v over the level bits; the input resident on
    the device.  CPU baseline: the reference's levelWT WT() (byte symbols,
    OpenMP) and its rank_support_v constructor on the same text."""
    import datagen
    n, L = 1 << log2_n, 8
    sym = datagen.zipf_bytes(n, seed=SEED + 29)
    d = torch.from_numpy(sym).to(dev)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    torch.cuda.synchronize()
    t = None
    for _ in range(3):
        t = wtg.WaveletTree.from_device(d.data_ptr(), n, 1, L, wtg.RANK, sp, tree=t)
    t.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        t = wtg.WaveletTree.from_device(d.data_ptr(), n, 1, L, wtg.RANK, sp, tree=t)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nb = n * L
    step_bytes = L * n + (L - 1) * n + nb / 8 + nb / 8 + 16 * ((nb >> 9) + 1)
    t.free()
    res = {"workload": f"byte text, n=2^{log2_n} uint8, Zipf(1.0) over 256 byte values, 8 levels, rank_support_v",
           "n": n, "levels": L, "ms": ms, "gbs": step_bytes / (ms / 1e3) / 1e9, "algorithmic_bytes": step_bytes,
           "cpu_baseline": None}
    if cpu:
        from oracle import oracle as O
        if O.ref_bench() is not None:
            t_wt, t_r = O.ref_bench_byte_text(sym, L)
            res["cpu_baseline"] = {"value": step_bytes / (t_wt + t_r) / 1e9, "unit": "GB/s",
                                   "cores": O.num_threads(), "kind": "reference",
                                   "sample": "the whole text: the reference's levelWT WT() (byte symbols) and "
                                             "rank_support_v constructor, OpenMP", "wt_s": t_wt, "rank_s": t_r}
    return res


LSEL_CONFIGS = (1024, 65536)  # segments per level and polarity: the named model, and a larger one


def measure_select(torch, wtg, tree, n, L, dev, stream, log2_q, reps=5, cpu_log2=0):
    """Learned select against plain select_support_mcl on the tree's levels:
    2^log2_q select1 and 2^log2_q select0 queries per pass (uniform level,
    uniform k), every learned answer compared with the plain one.  The first
    learned model is the named one (1024 segments); the second trades model
    space for narrower windows."""
    sp = stream.cuda_stream
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    nq = 1 << log2_q
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + 7)
    qs, outs = {}, {}
    bits = n * L

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    learned = []
    plain_ms = None
    exact = True
    for segs in LSEL_CONFIGS:
        b0, b1 = ev(), ev()
        b0.record(stream)
        ls = wtg.LearnedSelect(tree, segments=segs, samples=1024, max_window=1 << 16)
        b1.record(stream)
        torch.cuda.synchronize()
        info = ls.info()
        if not qs:
            for t_b in (1, 0):
                m_levels = [ls.level_model(t_b, l)[0]["m"] for l in range(L)]
                qs[t_b] = select_queries(torch, m_levels, nq, gen, dev)
                outs[t_b] = torch.empty(nq, device=dev, dtype=torch.int64)
                outs[("l", t_b)] = torch.empty(nq, device=dev, dtype=torch.int64)

            def run_plain():
                for t_b in (1, 0):
                    lv, k = qs[t_b]
                    tree.level_select_device(t_b, lv.data_ptr(), k.data_ptr(), nq, outs[t_b].data_ptr(), sp)
            plain_ms = timed(run_plain)

        def run_learned():
            for t_b in (1, 0):
                lv, k = qs[t_b]
                ls.select_device(t_b, lv.data_ptr(), k.data_ptr(), nq, outs[("l", t_b)].data_ptr(), sp)
        ms = timed(run_learned)
        ok = all(torch.equal(outs[t_b], outs[("l", t_b)]) for t_b in (1, 0))
        ok = ok and all(int((outs[t_b] == -1).sum().item()) == 0 for t_b in (1, 0))
        exact = exact and ok
        learned.append({
            "segments_per_level": segs, "mqs": 2 * nq / (ms / 1e3) / 1e6, "ms": ms, "speedup": plain_ms / ms,
            "exact": bool(ok), "space_bits_per_bit": 8 * info["index_bytes"] / bits,
            "index_bytes": info["index_bytes"], "segments": info["segments"],
            "fallback_segments": info["fallback_segments"], "max_window": info["max_window"],
            "mean_window": info["window_sum"] / max(1, info["segments"] - info["fallback_segments"]),
            "misses": info["misses"], "build_ms": b0.elapsed_time(b1),
        })
        ls.free()
    sel_tables = [tree.select_tables(t_b) for t_b in (0, 1)]
    mcl_words = sum(s.sb_nwords + s.nsb + s.pool_nwords for s in sel_tables)
    cpu = select_cpu_baseline(cpu_log2) if cpu_log2 else None
    return {
        "queries_per_pass": 2 * nq, "query_mix": f"2^{log2_q} select1 + 2^{log2_q} select0, uniform level and k",
        "plain_mqs": 2 * nq / (plain_ms / 1e3) / 1e6, "plain_ms": plain_ms,
        "learned_mqs": learned[0]["mqs"], "speedup": learned[0]["speedup"], "exact": bool(exact),
        "model": "piecewise-linear per level and polarity, least squares on 1024 pairs per segment, "
                 "exact error windows searched through rank_support_v",
        "mcl_space_bits_per_bit": 64 * mcl_words / bits,
        "learned": learned,
        "cpu_baseline": cpu,
    }


def select_cpu_baseline(log2_n, log2_q=22):
    """The reference's select_support_mcl<1>/<0>::select on the host cores
    (OpenMP over the queries) over the 20 levels of a 2^log2_n-symbol sample
    of the workload: 2^log2_q uniform select1 and select0 queries on the
    concatenated level bitvector, answers checked against the oracle."""
    import datagen
    from oracle import oracle as O
    if O.ref_bench() is None:
        return None
    n = 1 << log2_n
    sym = datagen.exp_u32(n, mean=MEAN, cap=CAP, seed=SEED)
    w, _ = O.wt_build(sym, LEVELS, tail=True)
    size = n * LEVELS
    ones = int(O.rank_build(w, size)[-2])
    rng = np.random.default_rng(SEED + 3)
    secs, nq = 0.0, 0
    for t_b, m in ((1, ones), (0, size - ones)):
        q = rng.integers(1, m + 1, 1 << log2_q).astype(np.uint64)
        dt, ans = O.ref_bench_select(w, size, t_b, q)
        if not np.array_equal(ans[:4096], O.Select(w, size, t_b).query_batch(q[:4096])):
            raise RuntimeError("reference select disagrees with the oracle")
        secs += dt
        nq += q.size
    return {"value": nq / secs / 1e6, "unit": "Mq/s", "cores": O.num_threads(), "kind": "reference",
            "sample": f"select_support_mcl<1>/<0>::select over the 20 x 2^{log2_n} level bits of a 2^{log2_n}-symbol "
                      f"sample, 2^{log2_q} uniform select1 + 2^{log2_q} select0 queries, OpenMP over queries"}


def run_wtg(args, rank, world, local_rank):
    import torch
    import wtg

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        init_ranks(dist, "nccl", args.rank_timeout)
    dev = torch.device("cuda", local_rank)
    n = 1 << args.n_log2
    L = LEVELS
    wtg.lib()

    # input, generated on the device (seeded per rank), then resident in HBM
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + rank)
    x = torch.empty(n, device=dev, dtype=torch.float32)
    x.exponential_(1.0 / MEAN, generator=g)
    seq = torch.clamp(torch.floor(x), max=CAP).to(torch.int32)
    del x
    torch.cuda.synchronize()

    # ---- e2e first, in a fresh process state: the host API from pinned host
    # buffers, the input copied in and every output copied back per step
    e2e = None
    if not args.no_e2e:
        import ctypes
        host_in = torch.empty(n, dtype=torch.int32, pin_memory=True)
        host_in.copy_(seq)
        h = ctypes.c_void_p()
        L_ = wtg.lib()
        wtg._ck(L_.wtg_tree_build(ctypes.c_void_p(host_in.data_ptr()), n, 4, L, wtg.ALL, ctypes.byref(h)))
        t_e = wtg.WaveletTree(_handle=h)
        s1, s0 = t_e.select_tables(1), t_e.select_tables(0)
        e2e_bytes = algorithmic_bytes(n, L, 4, sum(s.sb_nwords + s.nsb + s.pool_nwords for s in (s1, s0)))
        outs = {
            "bits": torch.empty(t_e.bit_words, dtype=torch.int64, pin_memory=True),
            "rank": torch.empty(t_e.rank_words, dtype=torch.int64, pin_memory=True),
        }
        for tb, s in ((1, s1), (0, s0)):
            outs[f"sb{tb}"] = torch.empty(max(s.sb_nwords, 1), dtype=torch.int64, pin_memory=True)
            outs[f"desc{tb}"] = torch.empty(max(s.nsb, 1), dtype=torch.int64, pin_memory=True)
            outs[f"pool{tb}"] = torch.empty(max(s.pool_nwords, 1), dtype=torch.int64, pin_memory=True)
        d2h = 8 * (t_e.bit_words + t_e.rank_words + sum(s.sb_nwords + s.nsb + s.pool_nwords for s in (s1, s0)))
        vp = ctypes.c_void_p

        def e2e_step():
            # bits and rank table come back while the build runs; then the
            # select tables (their sizes are known only after the build)
            wtg._ck(L_.wtg_tree_build_out(vp(host_in.data_ptr()), n, 4, L, wtg.ALL, vp(outs["bits"].data_ptr()),
                                          vp(outs["rank"].data_ptr()), ctypes.byref(h)))
            for tb in (1, 0):
                wtg._ck(L_.wtg_tree_get_select(h, tb, vp(outs[f"sb{tb}"].data_ptr()),
                                               vp(outs[f"desc{tb}"].data_ptr()), vp(outs[f"pool{tb}"].data_ptr())))

        for _ in range(max(1, args.warmup)):
            e2e_step()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e_steps = max(1, args.steps)
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(e_steps):
            ts = time.perf_counter()
            e2e_step()
            step_ms.append(1e3 * (time.perf_counter() - ts))
        torch.cuda.synchronize()
        e_s = slowest_rank(dist, torch, time.perf_counter() - t0, dev)
        e2e = {"value": job_throughput(world, e_steps, e2e_bytes, e_s), "unit": "GB/s",
               "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e_s / e_steps,
               "median_ms_per_step": round(float(np.median(step_ms)), 3), "step_ms": [round(x, 2) for x in step_ms]}
        t_e.free()
        del outs, host_in, t_e
        torch.cuda.empty_cache()

    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    tree = None
    for _ in range(args.warmup):
        tree = wtg.WaveletTree.from_device(seq.data_ptr(), n, 4, L, wtg.ALL, sp, tree=tree)
    torch.cuda.synchronize()
    tree.sync()

    sel = [tree.select_tables(t_b) for t_b in (0, 1)]
    sel_words = sum(s.sb_nwords + s.nsb + s.pool_nwords for s in sel)
    step_bytes = algorithmic_bytes(n, L, 4, sel_words)

    # ---- timed region: device-resident input
    wtg.profile_read()
    wtg.profile_enable(True)
    launches0 = wtg.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            tree = wtg.WaveletTree.from_device(seq.data_ptr(), n, 4, L, wtg.ALL, sp, tree=tree)
        end.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    tree.sync()
    launches = wtg.launch_count() - launches0
    wtg.profile_enable(False)
    prof = wtg.profile_read()
    ms = slowest_rank(dist, torch, start.elapsed_time(end), dev)
    value = job_throughput(world, args.steps, step_bytes, ms / 1e3)

    peak, peak_kind = measured_peaks()
    lv_n, lv_ms = prof["level"]
    lv_avg = lv_ms / max(lv_n, 1)
    lv_bytes = level_launch_bytes(n, 4)
    traffic = args.traffic if args.traffic is not None else LEVEL_DRAM_BYTES_PER_SYMBOL_U32 * n
    roofline = {
        "bound": "hbm", "kernel": "level_kernel<uint32,partition>", "achieved": lv_bytes / (lv_avg / 1e3) / 1e9,
        "peak": peak, "unit": "GB/s", "peak_kind": peak_kind, "traffic": traffic,
        "launch_ms": lv_avg, "launches": lv_n, "bytes_per_launch": lv_bytes,
    }
    roofline["frac"] = roofline["achieved"] / peak
    kernel_share = {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()}

    select = queries = batch = byte_text = None
    cpu_on = not args.no_cpu and rank == 0
    if cpu_on:
        from oracle import oracle as O
        O.build(ref=True)
    if not args.no_select:
        select = measure_select(torch, wtg, tree, n, L, dev, stream, args.select_log2,
                                cpu_log2=24 if cpu_on else 0)
        queries = measure_queries(torch, tree, seq, n, dev, stream, args.select_log2)
    if args.batch_texts:
        shape = tuple(int(x) for x in args.batch_shape.split(",")) if args.batch_shape else None
        batch = measure_batch(torch, wtg, stream, args.batch_texts, cpu_texts=512 if cpu_on else 0, shape=shape)
    if args.bytes_log2:
        byte_text = measure_byte_text(torch, wtg, dev, args.bytes_log2, cpu=cpu_on)
    fm = None
    if args.fm_log2:
        orc = None
        if not args.no_cpu:
            from oracle import oracle as orc
            orc.build(ref=False)
        fm = measure_fm(torch, wtg, orc, dev, args.fm_log2, args.fm_queries_log2, args.fm_cpu_log2)

    if rank != 0:
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        O.build(ref=True)
        cn = 1 << args.cpu_log2
        r = cpu_reference_seconds(cn)
        if r is not None:
            dt, b, cores = r
            cpu = {"value": b / dt / 1e9, "unit": "GB/s", "cores": cores, "kind": "reference",
                   "sample": f"n=2^{args.cpu_log2} of the same distribution, 20 levels, one full build ({dt:.2f} s) "
                             "by the reference's levelWT WT() + rank_support_v_par + select_support_mcl_par, OpenMP"}
        dt, b, cores = cpu_build_seconds(cn)
        port = {"value": b / dt / 1e9, "unit": "GB/s", "cores": cores, "kind": "port",
                "sample": f"n=2^{args.cpu_log2} of the same distribution, 20 levels, one full build ({dt:.2f} s) "
                          "by the oracle's restatement, OpenMP"}
        if cpu is None:
            cpu = port
        else:
            cpu["port"] = port

    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(n, world),
        "algorithmic_bytes_per_step": step_bytes,
        "hbm_frac": value / peak,
        "roofline": roofline,
        "kernel_time": kernel_share,
        "select": select,
        "queries": queries,
        "fm": fm,
        "batch": batch,
        "byte_text": byte_text,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wtg", choices=["wtg", "reference"])
    ap.add_argument("--n-log2", type=int, default=30)
    ap.add_argument("--cpu-log2", type=int, default=25,
                    help="log2 of the CPU baseline's sample (the reference arm: at most 26)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-select", action="store_true")
    ap.add_argument("--fm-log2", type=int, default=28,
                    help="FM-index core (suffix array, BWT, tree, counts) on a 2^k DNA text; 0 skips")
    ap.add_argument("--fm-queries-log2", type=int, default=24)
    ap.add_argument("--fm-cpu-log2", type=int, default=22)
    ap.add_argument("--bytes-log2", type=int, default=24,
                    help="byte-text build (Zipf bytes, 8 levels, rank) of 2^k symbols; 0 skips")
    ap.add_argument("--rank-timeout", type=float, default=600,
                    help="seconds a collective waits for the other ranks before it fails")
    ap.add_argument("--batch-shape", default=None,
                    help="fix the batch's shape as tile,whole_max,symbols_per_thread (default: autotuned)")
    ap.add_argument("--batch-texts", type=int, default=4096,
                    help="texts of the batched-build comparison (0: skip it)")
    ap.add_argument("--select-log2", type=int, default=26,
                    help="log2 of the select1 (and of the select0) queries per pass")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per level launch from an ncu capture, reported as roofline.traffic "
                         "(default: the n=2^26 capture scaled to n)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        args.cpu_log2 = min(args.cpu_log2, 26)
        run_reference(args, rank)
    else:
        run_wtg(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
