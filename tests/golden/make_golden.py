"""Generate the golden vectors in tests/golden/ from an independent restatement.

The reference (Rust) cannot be built or imported here and its tests hold no
known-answer vectors, so these fixtures come from a second, independent
restatement of the same published algorithms in pure Python big-integer
arithmetic (no code shared with the C oracle or the CUDA library):

  - KoalaBear Montgomery arithmetic and BinomialExtensionField<_, 4>, W = 3
  - the two-adic generators (from 3^127) and a naive O(n^2) DFT
  - ChaCha12 keyed by rand_core's PCG32 seed_from_u64 expansion, and the
    StandardUniform<KoalaBear> rejection sampler (next_u32 >> 1, < p)
  - Poseidon2 (MDSMat4 light layer, 1 1^T + diag internal layer, x^3, rounds
    (8,20) / (8,23), constants from StdRng(1000) as new_from_rng_128 draws them)
  - PaddingFreeSponge<P24,24,16,8>, TruncatedPermutation<P16,2,8,16>, the
    halves-paired Merkle tree, DuplexChallenger<F,P16,16,8>
  - the WHIR parameter formulas (crates/whir/src/params.rs)

plus the RFC 7539 section 2.3.2 ChaCha20 block test vector, which pins the
block function itself.  Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

P = 0x7F000001
R = (1 << 32) % P
RINV = pow(R, -1, P)
HERE = os.path.dirname(os.path.abspath(__file__))


def mont(x):
    return x % P * R % P


def unmont(a):
    return a * RINV % P


# ---------------- ChaCha / StdRng ----------------
def rotl(x, n):
    return ((x << n) | (x >> (32 - n))) & 0xFFFFFFFF


def chacha_block(key, counter, stream, rounds):
    s = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574] + list(key) + [
        counter & 0xFFFFFFFF, counter >> 32, stream & 0xFFFFFFFF, stream >> 32]
    x = list(s)

    def qr(a, b, c, d):
        x[a] = (x[a] + x[b]) & 0xFFFFFFFF; x[d] = rotl(x[d] ^ x[a], 16)
        x[c] = (x[c] + x[d]) & 0xFFFFFFFF; x[b] = rotl(x[b] ^ x[c], 12)
        x[a] = (x[a] + x[b]) & 0xFFFFFFFF; x[d] = rotl(x[d] ^ x[a], 8)
        x[c] = (x[c] + x[d]) & 0xFFFFFFFF; x[b] = rotl(x[b] ^ x[c], 7)

    for _ in range(rounds // 2):
        qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
        qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
    return [(a + b) & 0xFFFFFFFF for a, b in zip(x, s)]


def pcg32_key(state):
    MUL, INC, M64 = 6364136223846793005, 11634580027462260723, (1 << 64) - 1
    key = []
    for _ in range(8):
        state = (state * MUL + INC) & M64
        xs = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
        rot = state >> 59
        key.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF)
    return key


class StdRng:
    def __init__(self, seed):
        self.key = pcg32_key(seed)
        self.counter = 0
        self.buf = []

    def next_u32(self):
        if not self.buf:
            self.buf = chacha_block(self.key, self.counter, 0, 12)
            self.counter += 1
        return self.buf.pop(0)

    def field(self):  # Montgomery word
        while True:
            v = self.next_u32() >> 1
            if v < P:
                return v


# ---------------- Poseidon2 (on canonical values) ----------------
def frac(sign, num, log_den):
    v = num * pow(pow(2, log_den, P), -1, P) % P
    return (-v) % P if sign < 0 else v


V16 = [(-1, 2, 0), (1, 1, 0), (1, 2, 0), (1, 1, 1), (1, 3, 0), (1, 4, 0), (-1, 1, 1), (-1, 3, 0),
       (-1, 4, 0), (1, 1, 8), (1, 1, 3), (1, 1, 24), (-1, 1, 8), (-1, 1, 3), (-1, 1, 4),
       (-1, 1, 24)]
V24 = [(-1, 2, 0), (1, 1, 0), (1, 2, 0), (1, 1, 1), (1, 3, 0), (1, 4, 0), (-1, 1, 1), (-1, 3, 0),
       (-1, 4, 0), (1, 1, 8), (1, 1, 2), (1, 1, 3), (1, 1, 4), (1, 1, 5), (1, 1, 6), (1, 1, 24),
       (-1, 1, 8), (-1, 1, 3), (-1, 1, 4), (-1, 1, 5), (-1, 1, 6), (-1, 1, 7), (-1, 1, 9),
       (-1, 1, 24)]


def p2_consts(width):
    rp = 20 if width == 16 else 23
    rng = StdRng(1000)
    ext = [[unmont(rng.field()) for _ in range(width)] for _ in range(8)]
    intr = [unmont(rng.field()) for _ in range(rp)]
    diag = [frac(*v) for v in (V16 if width == 16 else V24)]
    return ext, intr, diag


def mds_light(s):
    w = len(s)
    for i in range(0, w, 4):
        x0, x1, x2, x3 = s[i:i + 4]
        s[i:i + 4] = [(2 * x0 + 3 * x1 + x2 + x3) % P, (x0 + 2 * x1 + 3 * x2 + x3) % P,
                      (x0 + x1 + 2 * x2 + 3 * x3) % P, (3 * x0 + x1 + x2 + 2 * x3) % P]
    sums = [sum(s[j] for j in range(c, w, 4)) % P for c in range(4)]
    return [(s[i] + sums[i % 4]) % P for i in range(w)]


CONSTS = {}


def permute(state_mont):
    w = len(state_mont)
    if w not in CONSTS:
        CONSTS[w] = p2_consts(w)
    ext, intr, diag = CONSTS[w]
    s = mds_light([unmont(v) for v in state_mont])
    for r in range(4):
        s = mds_light([pow((x + c) % P, 3, P) for x, c in zip(s, ext[r])])
    for c in intr:
        s[0] = pow((s[0] + c) % P, 3, P)
        tot = sum(s) % P
        s = [(tot + d * x) % P for x, d in zip(s, diag)]
    for r in range(4, 8):
        s = mds_light([pow((x + c) % P, 3, P) for x, c in zip(s, ext[r])])
    return [mont(x) for x in s]


def hash_leaf(row):
    s = [0] * 24
    pos, n = 0, len(row)
    while True:
        i = 0
        while i < 16 and pos < n:
            s[i] = row[pos]; i += 1; pos += 1
        if i == 16:
            s = permute(s)
            if pos == n:
                break
            continue
        if i:
            s = permute(s)
        break
    return s[:8]


def compress(l, r):
    return permute(list(l) + list(r))[:8]


def merkle_root(rows):
    layer = [hash_leaf(r) for r in rows]
    while len(layer) > 1:
        h = len(layer) // 2
        layer = [compress(layer[i], layer[i + h]) for i in range(h)]
    return layer[0]


# ---------------- field, extension, DFT ----------------
def ext_mul_c(a, b):  # canonical coefficient lists
    t = [0] * 7
    for i in range(4):
        for j in range(4):
            t[i + j] += a[i] * b[j]
    return [(t[0] + 3 * t[4]) % P, (t[1] + 3 * t[5]) % P, (t[2] + 3 * t[6]) % P, t[3] % P]


def two_adic(bits):
    return pow(3, 127 * (1 << (24 - bits)), P)


def dft_naive(rows_can, log_h):  # rows x width canonical, zero-padded
    h = 1 << log_h
    w = pow(3, 127 * (1 << (24 - log_h)), P) if log_h else 1
    width = len(rows_can[0])
    out = []
    for i in range(h):
        wi = pow(w, i, P)
        acc = [0] * width
        x = 1
        for r in rows_can:
            for c in range(width):
                acc[c] = (acc[c] + r[c] * x) % P
            x = x * wi % P
        out.append(acc)
    return out


# ---------------- challenger ----------------
class Challenger:
    def __init__(self):
        self.state = [0] * 16
        self.inp, self.out = [], []

    def duplex(self):
        for i, v in enumerate(self.inp):
            self.state[i] = v
        self.inp = []
        self.state = permute(self.state)
        self.out = self.state[:8]

    def observe(self, v):
        self.out = []
        self.inp.append(v)
        if len(self.inp) == 8:
            self.duplex()

    def sample(self):
        if self.inp or not self.out:
            self.duplex()
        return self.out.pop()


# ---------------- params (crates/whir/src/params.rs) ----------------
LOG2_10 = 3.321928094887362


def log_eta(s, lir):
    return 0.0 if s == 0 else (-(0.5 * lir + LOG2_10 + 1.0) if s == 1 else -(lir + LOG2_10 + 1.0))


def n_stir(s, sec, lir):
    eta = 2.0 ** log_eta(s, lir)
    rate = 1.0 / (1 << lir)
    delta = 0.5 * (1 - rate) if s == 0 else (1 - math.sqrt(rate) - eta if s == 1 else 1 - rate - eta)
    return math.ceil(-sec / math.log2(1 - delta))


def n_ood(s, sec, logd, lir, bits=124):
    if s == 0:
        return 0
    le = log_eta(s, lir)
    lsb = lir / 2 - (1 + le) if s == 1 else (logd + lir) - le
    for n in range(1, 64):
        if n * bits + 1 - (2 * lsb + logd * n) >= sec:
            return n
    return -1


def main():
    rng = StdRng(42)
    g = {}
    # field
    pairs = [(rng.field(), rng.field()) for _ in range(64)]
    g["fe_mul"] = [[a, b, mont(unmont(a) * unmont(b))] for a, b in pairs]
    g["fe_inv"] = [[a, mont(pow(unmont(a), P - 2, P))] for a, _ in pairs[:16] if a]
    g["two_adic_mont"] = [mont(two_adic(b)) for b in range(25)]
    exts = [[rng.field() for _ in range(4)] for _ in range(32)]
    g["ext_mul"] = [[a, b, [mont(x) for x in ext_mul_c([unmont(v) for v in a],
                                                       [unmont(v) for v in b])]]
                    for a, b in zip(exts[::2], exts[1::2])]
    # rng
    r1 = StdRng(1)
    g["rand_fe_seed1_first64"] = [r1.field() for _ in range(64)]
    g["chacha20_rfc7539"] = {
        "key": [0x03020100, 0x07060504, 0x0B0A0908, 0x0F0E0D0C, 0x13121110, 0x17161514,
                0x1B1A1918, 0x1F1E1D1C],
        "counter": (0x09000000 << 32) | 1, "stream": 0x4A000000,
        "out": [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3, 0xC7F4D1C7, 0x0368C033,
                0x9AAA2204, 0x4E6CD4C3, 0x466482D2, 0x09AA9F07, 0x05D7C214, 0xA2028BD9,
                0xD19C12B5, 0xB94E16DE, 0xE883D0CB, 0x4E3C50A2]}
    g["chacha12_seed1000_block0"] = chacha_block(pcg32_key(1000), 0, 0, 12)
    # poseidon2
    g["p2_16"] = [[s, permute(s)] for s in [list(range(16))] +
                  [[rng.field() for _ in range(16)] for _ in range(3)]]
    g["p2_24"] = [[s, permute(s)] for s in [list(range(24))] +
                  [[rng.field() for _ in range(24)] for _ in range(3)]]
    g["p2_constants_16"] = [[mont(x) for x in row] for row in CONSTS[16][0]] + \
        [[mont(x) for x in CONSTS[16][1]], [mont(x) for x in CONSTS[16][2]]]
    g["p2_constants_24"] = [[mont(x) for x in row] for row in CONSTS[24][0]] + \
        [[mont(x) for x in CONSTS[24][1]], [mont(x) for x in CONSTS[24][2]]]
    g["sponge"] = [[row, hash_leaf(row)] for row in
                   [[], [rng.field()], [rng.field() for _ in range(16)],
                    [rng.field() for _ in range(17)], [rng.field() for _ in range(64)]]]
    l, r = [rng.field() for _ in range(8)], [rng.field() for _ in range(8)]
    g["compress"] = [l, r, compress(l, r)]
    rows = [[rng.field() for _ in range(4)] for _ in range(8)]
    g["merkle"] = {"rows": rows, "root": merkle_root(rows)}
    # DFT
    cases = []
    for log_h, width, h_in in ((0, 2, 1), (2, 3, 4), (4, 2, 4), (5, 4, 8)):
        rws = [[rng.field() for _ in range(width)] for _ in range(h_in)]
        out = dft_naive([[unmont(v) for v in rr] for rr in rws], log_h)
        cases.append({"log_h": log_h, "width": width, "h_in": h_in, "in": rws,
                      "out": [[mont(v) for v in rr] for rr in out]})
    g["dft"] = cases
    # challenger: observe 0..n then sample, mixed
    ch = Challenger()
    seq = []
    for i in range(20):
        if i % 3 == 2:
            seq.append(["sample", ch.sample()])
        else:
            v = rng.field()
            ch.observe(v)
            seq.append(["observe", v])
    seq.append(["sample", ch.sample()])
    g["challenger"] = seq
    # params
    g["params"] = [[s, sec, logd, lir, n_ood(s, sec, logd, lir), n_stir(s, sec, lir)]
                   for s in (0, 1, 2) for sec in (32, 100, 123) for logd in (8, 16, 20, 24)
                   for lir in (1, 2, 3, 5)]
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
