"""ctypes wrapper of the C oracle (test infrastructure).

The oracle is a CPU restatement of the kilic/whir prover and verifier used
only as the correctness checker in tests/, in __graft_entry__.smoke() and as
the timed CPU baseline in bench.py.  Product code never imports this module.
Parity against the Rust reference itself is unpinned (the reference cannot be
built in this environment and its tests hold no golden vectors).
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwhir_oracle.so")

P = 0x7F000001
SOUNDNESS = {"UniqueDecoding": 0, "JohnsonBound": 1, "CapacityBound": 2}


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _bind(_lib)
    return _lib


u32p = ctypes.POINTER(ctypes.c_uint32)


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ("k", "folding", "rate", "initial_reduction", "soundness", "security_level")]


class Claims(ctypes.Structure):
    _fields_ = [("n_polys", ctypes.c_int), ("poly_k", ctypes.POINTER(ctypes.c_int)),
                ("n_groups", ctypes.c_int), ("group_n", ctypes.POINTER(ctypes.c_int)),
                ("group_ids", ctypes.POINTER(ctypes.c_int))]


def _bind(L):
    c = ctypes
    sig = {
        "wo_fe_from_u32": (c.c_uint32, [c.c_uint32]),
        "wo_fe_to_u32": (c.c_uint32, [c.c_uint32]),
        "wo_fe_mul": (c.c_uint32, [c.c_uint32, c.c_uint32]),
        "wo_set_packed": (None, [c.c_int]),
        "wo_fe_add": (c.c_uint32, [c.c_uint32, c.c_uint32]),
        "wo_fe_inv": (c.c_uint32, [c.c_uint32]),
        "wo_ext_mul": (None, [u32p, u32p, u32p]),
        "wo_two_adic_generator": (c.c_uint32, [c.c_int]),
        "wo_chacha_block": (None, [u32p, c.c_uint64, c.c_uint64, c.c_int, u32p]),
        "wo_rand_fe": (None, [c.c_uint64, u32p, c.c_size_t]),
        "wo_p2_permute": (c.c_int, [c.c_int, u32p]),
        "wo_p2_constants": (c.c_int, [c.c_int, u32p, u32p, u32p, c.POINTER(c.c_int)]),
        "wo_hash_leaf": (None, [u32p, c.c_size_t, u32p]),
        "wo_compress": (None, [u32p, u32p, u32p]),
        "wo_dft_batch": (None, [u32p, c.c_size_t, c.c_size_t, c.c_int, u32p]),
        "wo_merkle_tree": (None, [u32p, c.c_int, c.c_size_t, u32p]),
        "wo_eq_table": (None, [u32p, c.c_int, u32p, u32p]),
        "wo_compress_hi": (None, [u32p, c.c_int, u32p, c.c_int, u32p]),
        "wo_compress_lo": (None, [u32p, c.c_int, u32p, c.c_int, u32p]),
        "wo_eval_ext": (None, [u32p, c.c_int, u32p, u32p]),
        "wo_coeffs": (None, [u32p, u32p, c.c_int, u32p, u32p]),
        "wo_fix_lo": (None, [u32p, c.c_int, u32p]),
        "wo_combine_eqs": (None, [u32p, c.c_int, u32p, c.c_int, u32p]),
        "wo_combine_pows": (None, [u32p, c.c_int, u32p, c.c_int, u32p, c.c_int]),
        "wo_combine_pows_scaled": (None, [u32p, c.c_int, u32p, c.c_int, u32p]),
        "wo_n_ood_queries": (c.c_int, [c.c_int] * 5),
        "wo_n_stir_queries": (c.c_int, [c.c_int] * 3),
        "wo_number_of_rounds": (None, [c.c_int, c.c_int, c.POINTER(c.c_int), c.POINTER(c.c_int)]),
        "wo_svo_accumulators": (None, [u32p, c.c_int, u32p, c.c_int, u32p]),
        "wo_prove": (c.c_int, [c.POINTER(Params), c.POINTER(Claims), u32p, c.c_char_p,
                               c.c_size_t, c.POINTER(c.c_size_t), u32p]),
        "wo_verify": (c.c_int, [c.POINTER(Params), c.POINTER(Claims), c.c_char_p, c.c_size_t,
                                u32p]),
        "wo_threads": (c.c_int, []),
        "wo_set_threads": (None, [c.c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def ptr(a):
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(u32p)


def rand_fe(seed, n):
    out = np.empty(n, np.uint32)
    lib().wo_rand_fe(seed, ptr(out), n)
    return out


def to_mont(x):
    x = np.asarray(x, dtype=np.uint64) % P
    return ((x << np.uint64(32)) % np.uint64(P)).astype(np.uint32)


def from_mont(x):
    x = np.asarray(x, dtype=np.uint64)
    rinv = pow(2 ** 32, -1, P)
    return ((x * np.uint64(rinv)) % np.uint64(P)).astype(np.uint32)


def p2_permute(width, state):
    s = np.ascontiguousarray(state, dtype=np.uint32).copy()
    assert lib().wo_p2_permute(width, ptr(s)) == 0
    return s


def p2_constants(width):
    ext = np.empty(8 * width, np.uint32)
    intr = np.empty(32, np.uint32)
    diag = np.empty(width, np.uint32)
    rp = ctypes.c_int()
    assert lib().wo_p2_constants(width, ptr(ext), ptr(intr), ptr(diag), ctypes.byref(rp)) == 0
    return ext, intr[: rp.value].copy(), diag


def dft_batch(inp, h_in, width, log_h):
    inp = np.ascontiguousarray(inp, dtype=np.uint32)
    out = np.empty((1 << log_h) * width, np.uint32)
    lib().wo_dft_batch(ptr(inp), h_in, width, log_h, ptr(out))
    return out


def merkle_tree(rows, log_h, row_len):
    rows = np.ascontiguousarray(rows, dtype=np.uint32)
    out = np.empty(((2 << log_h) - 1) * 8, np.uint32)
    lib().wo_merkle_tree(ptr(rows), log_h, row_len, ptr(out))
    return out


def hash_leaf(row):
    row = np.ascontiguousarray(row, dtype=np.uint32)
    out = np.empty(8, np.uint32)
    lib().wo_hash_leaf(ptr(row), row.size, ptr(out))
    return out


def compress(left, right):
    out = np.empty(8, np.uint32)
    lib().wo_compress(ptr(np.ascontiguousarray(left, np.uint32)),
                      ptr(np.ascontiguousarray(right, np.uint32)), ptr(out))
    return out


def ext_one():
    return np.array([to_mont(1), 0, 0, 0], np.uint32)


def eq_table(point, k, scale=None):
    scale = ext_one() if scale is None else np.ascontiguousarray(scale, np.uint32)
    out = np.empty((1 << k) * 4, np.uint32)
    lib().wo_eq_table(ptr(np.ascontiguousarray(point, np.uint32)), k, ptr(scale), ptr(out))
    return out


def compress_hi(poly, k, point, kz):
    out = np.empty((1 << (k - kz)) * 4, np.uint32)
    lib().wo_compress_hi(ptr(poly), k, ptr(np.ascontiguousarray(point, np.uint32)), kz, ptr(out))
    return out


def compress_lo(poly, k, point, kz):
    out = np.empty((1 << (k - kz)) * 4, np.uint32)
    lib().wo_compress_lo(ptr(poly), k, ptr(np.ascontiguousarray(point, np.uint32)), kz, ptr(out))
    return out


def eval_ext(poly, k, point):
    out = np.empty(4, np.uint32)
    lib().wo_eval_ext(ptr(poly), k, ptr(np.ascontiguousarray(point, np.uint32)), ptr(out))
    return out


def coeffs(poly, weights, k):
    c0 = np.empty(4, np.uint32)
    c2 = np.empty(4, np.uint32)
    lib().wo_coeffs(ptr(poly), ptr(weights), k, ptr(c0), ptr(c2))
    return c0, c2


def fix_lo(poly, k, r):
    a = np.ascontiguousarray(poly, np.uint32).copy()
    lib().wo_fix_lo(ptr(a), k, ptr(np.ascontiguousarray(r, np.uint32)))
    return a[: (1 << (k - 1)) * 4].copy()


def combine_eqs(weights, k, points, n, alpha):
    w = np.ascontiguousarray(weights, np.uint32).copy()
    lib().wo_combine_eqs(ptr(w), k, ptr(np.ascontiguousarray(points, np.uint32)), n,
                         ptr(np.ascontiguousarray(alpha, np.uint32)))
    return w


def combine_pows(weights, k, vars_, n, alpha, shift):
    w = np.ascontiguousarray(weights, np.uint32).copy()
    lib().wo_combine_pows(ptr(w), k, ptr(np.ascontiguousarray(vars_, np.uint32)), n,
                          ptr(np.ascontiguousarray(alpha, np.uint32)), shift)
    return w


def combine_pows_scaled(weights, k, vars_, n, scales):
    w = np.ascontiguousarray(weights, np.uint32).copy()
    lib().wo_combine_pows_scaled(ptr(w), k, ptr(np.ascontiguousarray(vars_, np.uint32)), n,
                                 ptr(np.ascontiguousarray(scales, np.uint32)))
    return w


def n_ood_queries(soundness, security, log_degree, log_inv_rate, field_bits=124):
    return lib().wo_n_ood_queries(soundness, security, log_degree, log_inv_rate, field_bits)


def n_stir_queries(soundness, security, log_inv_rate):
    return lib().wo_n_stir_queries(soundness, security, log_inv_rate)


def number_of_rounds(folding, k):
    a, b = ctypes.c_int(), ctypes.c_int()
    lib().wo_number_of_rounds(folding, k, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def svo_accumulators(poly, k, point, l0):
    """SvoPoint::eval's claim value and Svo::calculate_accumulators with weight
    1: (value, accumulators), 4 words per extension element; per round r < l0,
    3^r entries at u_r = 0, then 3^r at u_r = 2."""
    n = sum(2 * 3 ** r for r in range(l0))
    out = np.zeros(4 + 4 * n, np.uint32)
    lib().wo_svo_accumulators(ptr(np.ascontiguousarray(poly, np.uint32)), k,
                              ptr(np.ascontiguousarray(point, np.uint32)), l0, ptr(out))
    return out[:4], out[4:]


def _claims(poly_ks, groups):
    n = len(poly_ks)
    pk = (ctypes.c_int * n)(*poly_ks)
    gn = (ctypes.c_int * max(1, len(groups)))(*[len(g) for g in groups])
    flat = [i for g in groups for i in g]
    gi = (ctypes.c_int * max(1, len(flat)))(*flat)
    cl = Claims(n, pk, len(groups), gn, gi)
    cl._keep = (pk, gn, gi)
    return cl


def prove(params, polys, poly_ks, groups, cap=None):
    """Prove like the reference harness; returns (proof bytes, checkpoint)."""
    prm = Params(*params)
    cl = _claims(poly_ks, groups)
    flat = np.ascontiguousarray(np.concatenate(polys), np.uint32)
    cap = cap or (64 << 20)
    buf = ctypes.create_string_buffer(cap)
    ln = ctypes.c_size_t()
    cp = np.zeros(1, np.uint32)
    rc = lib().wo_prove(ctypes.byref(prm), ctypes.byref(cl), ptr(flat), buf, cap,
                        ctypes.byref(ln), ptr(cp))
    if rc != 0:
        raise RuntimeError(f"oracle prove failed: {rc}")
    return buf.raw[: ln.value], int(cp[0])


def verify(params, poly_ks, groups, proof):
    prm = Params(*params)
    cl = _claims(poly_ks, groups)
    cp = np.zeros(1, np.uint32)
    rc = lib().wo_verify(ctypes.byref(prm), ctypes.byref(cl), proof, len(proof), ptr(cp))
    return rc, int(cp[0])


def set_packed(on):
    """Merkle hashing through the lane-packed permutation (the timed baseline);
    the results are the same as the scalar path's."""
    lib().wo_set_packed(1 if on else 0)
