"""Seeded synthetic inputs with the shapes and value distributions of the
workloads this library is measured on (the reference's own benchmark inputs,
Pizza&Chili corpora and PBBS sequence files, are not available offline).

  zipf_bytes       n uint8 symbols, Zipf(s) over 256 byte values, random
                   rank->byte permutation (byte text, 8 levels)
  dna_markov       n uint8 over {A,C,G,T,N}: order-2 Markov chain with
                   Dirichlet(1) transition rows, N forced in runs of 1-100 to
                   0.1% of positions
  exp_u32          n uint32, min(floor(Exp(mean)), cap) (integer tree,
                   sigma 2^20, 20 levels)
  batch_texts      k texts, lengths log-uniform in [2^lo, 2^hi], uniform ACGT
All generators are deterministic in `seed` (numpy PCG64).
"""
import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)
ACGTN = np.frombuffer(b"ACGNT", dtype=np.uint8)


def zipf_bytes(n, s=1.0, seed=0):
    rng = np.random.default_rng(seed)
    ranks = np.arange(1, 257, dtype=np.float64)
    p = ranks ** (-s)
    p /= p.sum()
    perm = rng.permutation(256).astype(np.uint8)
    out = np.empty(n, dtype=np.uint8)
    chunk = 1 << 24
    cdf = np.cumsum(p)
    cdf[-1] = 1.0
    for o in range(0, n, chunk):
        m = min(chunk, n - o)
        r = np.searchsorted(cdf, rng.random(m), side="right")
        out[o:o + m] = perm[np.minimum(r, 255)]
    return out


def exp_u32(n, mean=2 ** 14, cap=2 ** 20 - 1, seed=0):
    rng = np.random.default_rng(seed)
    out = np.empty(n, dtype=np.uint32)
    chunk = 1 << 24
    for o in range(0, n, chunk):
        m = min(chunk, n - o)
        v = np.floor(rng.exponential(mean, m))
        out[o:o + m] = np.minimum(v, cap).astype(np.uint32)
    return out


def dna_markov(n, seed=0, n_frac=0.001):
    rng = np.random.default_rng(seed)
    trans = rng.dirichlet(np.ones(4), size=16)  # context = previous two bases
    cdf = np.cumsum(trans, axis=1)
    cdf[:, -1] = 1.0
    codes = np.empty(n, dtype=np.uint8)
    if n == 0:
        return codes
    u = rng.random(n)
    a, b = rng.integers(0, 4), rng.integers(0, 4)
    # sequential chain; vectorised per block would change the distribution,
    # so run it in chunks with a small Python loop over the state
    for i in range(n):
        ctx = a * 4 + b
        c = int(np.searchsorted(cdf[ctx], u[i], side="right"))
        c = min(c, 3)
        codes[i] = c
        a, b = b, c
    text = ACGT[codes]
    target = int(round(n * n_frac))
    placed = 0
    while placed < target:
        ln = int(rng.integers(1, 101))
        st = int(rng.integers(0, max(1, n - ln)))
        seg = text[st:st + ln]
        placed += int(np.count_nonzero(seg != ord("N")))
        text[st:st + ln] = ord("N")
    return text


def dna_markov_device(n, torch, device, seed=0, n_frac=0.001, block=4096):
    """dna_markov's distribution generated on the GPU for large n: the text
    is cut into blocks of `block` symbols, each an order-2 chain from a
    uniform start (restarts cost a few symbols of mixing per block); N runs
    of U[1, 100] symbols until about n_frac of the text is N.  uint8 ACGTN."""
    rng = np.random.default_rng(seed)
    trans = rng.dirichlet(np.ones(4), size=16)
    cdf = torch.tensor(np.cumsum(trans, axis=1)[:, :3], dtype=torch.float32, device=device)
    nb = (n + block - 1) // block
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    a = torch.randint(0, 4, (nb,), device=device, generator=g)
    b = torch.randint(0, 4, (nb,), device=device, generator=g)
    codes = torch.empty((block, nb), dtype=torch.uint8, device=device)
    for i in range(block):
        u = torch.rand(nb, device=device, generator=g)
        row = cdf[a * 4 + b]
        c = (u.unsqueeze(1) > row).sum(dim=1)
        codes[i] = c.to(torch.uint8)
        a, b = b, c
    lut = torch.tensor(np.frombuffer(b"ACGT", np.uint8).copy(), device=device)
    text = lut[codes.t().reshape(-1)[:n].long()]
    runs = int(round(n * n_frac / 50.5))
    if runs:
        ln = torch.randint(1, 101, (runs,), device=device, generator=g)
        st = torch.randint(0, max(1, n - 100), (runs,), device=device, generator=g)
        idx = (st.unsqueeze(1) + torch.arange(100, device=device).unsqueeze(0))
        idx = idx[torch.arange(100, device=device).unsqueeze(0) < ln.unsqueeze(1)]
        text[idx] = ord("N")
    return text.contiguous()


def batch_texts(k=4096, lo=10, hi=20, seed=0):
    rng = np.random.default_rng(seed)
    lens = np.floor(2.0 ** rng.uniform(lo, hi, k)).astype(np.int64)
    return [ACGT[rng.integers(0, 4, int(m))] for m in lens]


def random_bits(size, density, seed=0):
    """uint64 words of a random bit_vector of `size` bits (bits past the end zero)."""
    rng = np.random.default_rng(seed)
    nw = (size + 63) // 64
    if nw == 0:
        return np.zeros(0, dtype=np.uint64)
    bits = rng.random(nw * 64) < density
    bits[size:] = False
    return np.packbits(bits.reshape(-1, 8), axis=1, bitorder="little").reshape(-1).view(np.uint64).copy()
