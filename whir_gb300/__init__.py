"""GB300-native WHIR prover: Python mirror of the C ABI in include/whir_gb300.h.

The compute path is libwhir_gb300.so (hand-written sm_103a CUDA kernels and a
C++ host); this module only binds it with ctypes and mirrors the reference's
prover interface (kilic/whir ``Whir::{new, commit, open}``, ``ProverStack``,
``PoseidonWriter``) so tests and benchmarks read like the reference's own.
There is no CPU fallback: every call fails loudly when the library or a GPU is
missing.

Field elements are numpy uint32 arrays of Montgomery words (Plonky3's
KoalaBear representation); an extension element is 4 words.
"""

import ctypes
import os

import numpy as np

from . import build as _build

P = 0x7F000001
SOUNDNESS = {"UniqueDecoding": 0, "JohnsonBound": 1, "CapacityBound": 2}
PROF_DFT, PROF_LEAF, PROF_TREE, PROF_SUMCHECK, PROF_SYNC = 0, 1, 2, 3, 4

_lib = None
u32p = ctypes.POINTER(ctypes.c_uint32)
i32p = ctypes.POINTER(ctypes.c_int32)
vp = ctypes.c_void_p


class WhirError(RuntimeError):
    pass


class Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("k", "folding", "rate", "initial_reduction", "soundness", "security_level")]


class JobC(ctypes.Structure):
    """struct whir_job (include/whir_gb300.h)."""
    _fields_ = [("params", Params), ("poly", ctypes.c_void_p), ("poly_on_device", ctypes.c_int32),
                ("n_claims", ctypes.c_int32), ("commit_only", ctypes.c_int32),
                ("arrival_s", ctypes.c_double), ("proof", ctypes.c_void_p),
                ("proof_cap", ctypes.c_size_t), ("proof_len", ctypes.c_size_t),
                ("checkpoint", ctypes.c_uint32), ("status", ctypes.c_int32),
                ("worker", ctypes.c_int32), ("start_s", ctypes.c_double),
                ("done_s", ctypes.c_double)]


class RunStatsC(ctypes.Structure):
    _fields_ = [("seconds", ctypes.c_double), ("peak_device_bytes", ctypes.c_uint64)]


_SIGS = {
    "whir_last_error": (ctypes.c_char_p, []),
    "whir_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(vp)]),
    "whir_ctx_destroy": (ctypes.c_int, [vp]),
    "whir_ctx_stream": (ctypes.c_int, [vp, ctypes.POINTER(vp)]),
    "whir_device_alloc": (ctypes.c_int, [vp, ctypes.c_size_t, ctypes.POINTER(vp)]),
    "whir_device_free": (ctypes.c_int, [vp, vp]),
    "whir_copy_to_device": (ctypes.c_int, [vp, vp, vp, ctypes.c_size_t]),
    "whir_copy_to_host": (ctypes.c_int, [vp, vp, vp, ctypes.c_size_t]),
    "whir_dft_batch": (ctypes.c_int, [vp, vp, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, vp]),
    "whir_merkle_commit": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_size_t,
                                          ctypes.POINTER(vp), u32p]),
    "whir_merkle_levels": (ctypes.c_int, [vp, u32p]),
    "whir_merkle_open": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_size_t), ctypes.c_size_t,
                                        u32p]),
    "whir_merkle_free": (ctypes.c_int, [vp]),
    "whir_eq_table": (ctypes.c_int, [vp, u32p, ctypes.c_int, u32p, vp]),
    "whir_compress_hi": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, ctypes.c_int, u32p]),
    "whir_compress_lo": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, ctypes.c_int, vp]),
    "whir_eval_ext": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, u32p]),
    "whir_sumcheck_coeffs": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, u32p, u32p]),
    "whir_sumcheck_fold": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, u32p, vp, vp]),
    "whir_combine_eqs": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, ctypes.c_int, u32p]),
    "whir_combine_pows": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, ctypes.c_int, u32p,
                                         ctypes.c_int]),
    "whir_combine_pows_scaled": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, ctypes.c_int, u32p]),
    "whir_transcript_new": (ctypes.c_int, [ctypes.POINTER(vp)]),
    "whir_transcript_free": (ctypes.c_int, [vp]),
    "whir_transcript_write": (ctypes.c_int, [vp, u32p]),
    "whir_transcript_write_base": (ctypes.c_int, [vp, ctypes.c_uint32]),
    "whir_transcript_draw": (ctypes.c_int, [vp, u32p]),
    "whir_transcript_draw_base": (ctypes.c_int, [vp, u32p]),
    "whir_transcript_draw_bits": (ctypes.c_int, [vp, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_size_t)]),
    "whir_transcript_size": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_size_t)]),
    "whir_transcript_bytes": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t]),
    "whir_prover_new": (ctypes.c_int, [vp, ctypes.POINTER(Params), ctypes.POINTER(vp)]),
    "whir_prover_free": (ctypes.c_int, [vp]),
    "whir_commit": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, i32p, ctypes.c_int]),
    "whir_stack_eval": (ctypes.c_int, [vp, vp, ctypes.c_int, u32p, u32p]),
    "whir_open": (ctypes.c_int, [vp, vp]),
    "whir_prove": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, i32p, ctypes.c_int, i32p,
                                  ctypes.c_int, i32p]),
    "whir_prof_enable": (ctypes.c_int, [vp, ctypes.c_int]),
    "whir_prof_enable_classes": (ctypes.c_int, [vp, ctypes.c_uint]),
    "whir_prof_read": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_long),
                                      ctypes.POINTER(ctypes.c_double)]),
    "whir_poseidon2_permute": (ctypes.c_int, [ctypes.c_int, u32p]),
    "whir_random_field": (ctypes.c_int, [ctypes.c_uint64, u32p, ctypes.c_size_t]),
    "whir_batch_prove": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(JobC), ctypes.c_int,
                                        ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(RunStatsC)]),
    "whir_serve": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(JobC), ctypes.c_int,
                                  ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(RunStatsC)]),
    "whir_autotune": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                     ctypes.c_size_t]),
    "whir_tune_tree": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "whir_tune_dft": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.c_int]),
    "whir_tune_reset": (ctypes.c_int, []),
    "whir_verify": (ctypes.c_int, [ctypes.POINTER(Params), i32p, ctypes.c_int, i32p, ctypes.c_int,
                                   i32p, ctypes.c_char_p, ctypes.c_size_t, i32p, u32p]),
    "whir_verify_batch": (ctypes.c_int, [vp, ctypes.POINTER(Params), i32p, ctypes.c_int, i32p,
                                         ctypes.c_int, i32p, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_void_p),
                                         ctypes.POINTER(ctypes.c_size_t), i32p, u32p]),
    "whir_server_new": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                       ctypes.POINTER(vp)]),
    "whir_server_run": (ctypes.c_int, [vp, ctypes.POINTER(JobC), ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(RunStatsC)]),
    "whir_server_free": (ctypes.c_int, [vp]),
    "whir_server_set_lockstep": (ctypes.c_int, [vp, ctypes.c_int]),
    "whir_workspace_bytes": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_uint64)]),
    "whir_proof_bytes_max": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_uint64)]),
    "whir_serve_simulate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                           ctypes.c_int, ctypes.c_uint64,
                                           ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double), i32p, i32p]),
    "whir_prove_batch": (ctypes.c_int, [vp, ctypes.POINTER(Params), ctypes.POINTER(vp),
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_char_p, ctypes.c_size_t,
                                        ctypes.POINTER(ctypes.c_size_t), u32p]),
    "whir_batch_max": (ctypes.c_int, [ctypes.POINTER(Params), i32p]),
    "whir_serve_simulate_groups": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_uint64),
                                                  ctypes.POINTER(ctypes.c_double), i32p,
                                                  ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_uint64,
                                                  ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double), i32p, i32p]),
    "whir_fold_code_rounds": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_size_t), ctypes.c_int, u32p,
                                             u32p, u32p, u32p]),
    "whir_debug_set": (ctypes.c_int, [ctypes.c_uint]),
    "whir_counters": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(ctypes.c_uint64),
                                     ctypes.POINTER(ctypes.c_uint64)]),
}


def lib_path():
    return _build.LIB


def lib():
    """Load libwhir_gb300.so (building it if absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            _build.build()
        L = ctypes.CDLL(_build.LIB)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        msg = lib().whir_last_error()
        raise WhirError(f"whir error {rc}: {msg.decode() if msg else ''}")


def _u32(a):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(u32p)


class DeviceArray:
    """Device allocation of the context's GPU (freed on close / GC)."""

    def __init__(self, ctx, nbytes):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = vp()
        _check(lib().whir_device_alloc(ctx.h, max(16, self.nbytes), ctypes.byref(p)))
        self.ptr = p.value

    def close(self):
        if self.ptr:
            lib().whir_device_free(self.ctx.h, self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        _check(lib().whir_copy_to_device(self.ctx.h, self.ptr, arr.ctypes.data, arr.nbytes))
        return self

    def download(self, n_words, dtype=np.uint32):
        out = np.empty(n_words, dtype)
        _check(lib().whir_copy_to_host(self.ctx.h, out.ctypes.data, self.ptr, out.nbytes))
        return out


class Context:
    """One GPU and one CUDA stream (whir_ctx)."""

    def __init__(self, device=0):
        h = vp()
        _check(lib().whir_ctx_create(device, ctypes.byref(h)))
        self.h = h.value

    def close(self):
        if self.h:
            lib().whir_ctx_destroy(self.h)
            self.h = None

    def stream(self):
        s = vp()
        _check(lib().whir_ctx_stream(self.h, ctypes.byref(s)))
        return s.value

    def alloc(self, nbytes):
        return DeviceArray(self, nbytes)

    def to_device(self, arr):
        arr = np.ascontiguousarray(arr)
        return DeviceArray(self, arr.nbytes).upload(arr)

    def prof_enable(self, on=True):
        _check(lib().whir_prof_enable(self.h, 1 if on else 0))

    def prof_enable_classes(self, classes):
        """Time only these classes (PROF_DFT, PROF_LEAF, ...)."""
        mask = 0
        for c in classes:
            mask |= 1 << c
        _check(lib().whir_prof_enable_classes(self.h, ctypes.c_uint(mask)))

    def counters(self):
        """(kernel launches in this process, prover h2d bytes, prover d2h bytes)"""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().whir_counters(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def prof_read(self, klass):
        ms, n, b = ctypes.c_double(), ctypes.c_long(), ctypes.c_double()
        _check(lib().whir_prof_read(self.h, klass, ctypes.byref(ms), ctypes.byref(n),
                                    ctypes.byref(b)))
        return ms.value, n.value, b.value


# ---- kernel-level entry points (device arrays in, numpy or device out) ----
def dft_batch(ctx, dev_in, h_in, width, log_h):
    out = ctx.alloc(4 * width << log_h)
    _check(lib().whir_dft_batch(ctx.h, dev_in.ptr, h_in, width, log_h, out.ptr))
    return out


class MerkleTree:
    def __init__(self, ctx, dev_rows, log_h, row_len):
        self.ctx, self.rows, self.log_h, self.row_len = ctx, dev_rows, log_h, row_len
        h = vp()
        root = np.zeros(8, np.uint32)
        _check(lib().whir_merkle_commit(ctx.h, dev_rows.ptr, log_h, row_len, ctypes.byref(h),
                                        root.ctypes.data_as(u32p)))
        self.h, self.root = h.value, root

    def levels(self):
        out = np.empty(((2 << self.log_h) - 1) * 8, np.uint32)
        _check(lib().whir_merkle_levels(self.h, out.ctypes.data_as(u32p)))
        return out

    def open(self, indexes):
        idx = np.ascontiguousarray(indexes, dtype=np.uintp)
        per = self.row_len + 8 * self.log_h
        out = np.empty(per * len(idx), np.uint32)
        _check(lib().whir_merkle_open(self.h, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_size_t)),
                                      len(idx), out.ctypes.data_as(u32p)))
        return out.reshape(len(idx), per)

    def close(self):
        if self.h:
            lib().whir_merkle_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eq_table(ctx, point, k, scale):
    out = ctx.alloc(16 << k)
    pt, pp = _u32(point)
    sc, sp = _u32(scale)
    _check(lib().whir_eq_table(ctx.h, pp, k, sp, out.ptr))
    return out


def compress_hi(ctx, dev_poly, k, point, kz):
    out = np.empty(4 << (k - kz), np.uint32)
    pt, pp = _u32(point)
    _check(lib().whir_compress_hi(ctx.h, dev_poly.ptr, k, pp, kz, out.ctypes.data_as(u32p)))
    return out


def compress_lo(ctx, dev_poly, k, point, kz):
    out = ctx.alloc(16 << (k - kz))
    pt, pp = _u32(point)
    _check(lib().whir_compress_lo(ctx.h, dev_poly.ptr, k, pp, kz, out.ptr))
    return out


def eval_ext(ctx, dev_poly, k, point):
    out = np.empty(4, np.uint32)
    pt, pp = _u32(point)
    _check(lib().whir_eval_ext(ctx.h, dev_poly.ptr, k, pp, out.ctypes.data_as(u32p)))
    return out


def sumcheck_coeffs(ctx, dev_poly, dev_w, k):
    c0, c2 = np.empty(4, np.uint32), np.empty(4, np.uint32)
    _check(lib().whir_sumcheck_coeffs(ctx.h, dev_poly.ptr, dev_w.ptr, k,
                                      c0.ctypes.data_as(u32p), c2.ctypes.data_as(u32p)))
    return c0, c2


def sumcheck_fold(ctx, dev_poly, dev_w, k, r):
    po, wo = ctx.alloc(16 << (k - 1)), ctx.alloc(16 << (k - 1))
    rr, rp = _u32(r)
    _check(lib().whir_sumcheck_fold(ctx.h, dev_poly.ptr, dev_w.ptr, k, rp, po.ptr, wo.ptr))
    return po, wo


def combine_eqs(ctx, dev_w, k, points, n, alpha):
    pt, pp = _u32(points)
    al, ap = _u32(alpha)
    _check(lib().whir_combine_eqs(ctx.h, dev_w.ptr, k, pp, n, ap))


def combine_pows(ctx, dev_w, k, vars_, n, alpha, shift):
    va, vpp = _u32(vars_)
    al, ap = _u32(alpha)
    _check(lib().whir_combine_pows(ctx.h, dev_w.ptr, k, vpp, n, ap, shift))


def combine_pows_scaled(ctx, dev_w, k, vars_, n, scales):
    va, vpp = _u32(vars_)
    sc, sp = _u32(scales)
    _check(lib().whir_combine_pows_scaled(ctx.h, dev_w.ptr, k, vpp, n, sp))


def random_field(seed, n, out=None):
    """Poly::rand(&mut rng(seed), ..): n seeded KoalaBear elements (Montgomery words)."""
    out = np.empty(n, np.uint32) if out is None else out
    _check(lib().whir_random_field(seed, out.ctypes.data_as(u32p), n))
    return out


def poseidon2_permute(width, state):
    s, sp = _u32(np.array(state, dtype=np.uint32).copy())
    _check(lib().whir_poseidon2_permute(width, sp))
    return s


# ---- transcript and protocol ----
class PoseidonWriter:
    """PoseidonWriter<Vec<u8>, KoalaBear, DuplexChallenger<_, Poseidon2<16>, 16, 8>>."""

    def __init__(self):
        h = vp()
        _check(lib().whir_transcript_new(ctypes.byref(h)))
        self.h = h.value

    def write(self, e):
        a, p = _u32(e)
        _check(lib().whir_transcript_write(self.h, p))

    def write_base(self, v):
        _check(lib().whir_transcript_write_base(self.h, int(v)))

    def draw(self):
        out = np.empty(4, np.uint32)
        _check(lib().whir_transcript_draw(self.h, out.ctypes.data_as(u32p)))
        return out

    def draw_base(self):
        out = np.empty(1, np.uint32)
        _check(lib().whir_transcript_draw_base(self.h, out.ctypes.data_as(u32p)))
        return int(out[0])

    def draw_bits(self, bits):
        out = ctypes.c_size_t()
        _check(lib().whir_transcript_draw_bits(self.h, bits, ctypes.byref(out)))
        return out.value

    def finalize(self):
        n = ctypes.c_size_t()
        _check(lib().whir_transcript_size(self.h, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(max(1, n.value))
        _check(lib().whir_transcript_bytes(self.h, buf, n.value))
        return buf.raw[: n.value]

    def close(self):
        if self.h:
            lib().whir_transcript_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Whir:
    """Whir::new(k, folding, rate, initial_reduction, soundness, security_level)."""

    def __init__(self, ctx, k, folding, rate, initial_reduction, soundness, security_level):
        self.ctx = ctx
        if isinstance(soundness, str):
            soundness = SOUNDNESS[soundness]
        self.params = Params(k, folding, rate, initial_reduction, soundness, security_level)
        h = vp()
        _check(lib().whir_prover_new(ctx.h, ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h.value

    @staticmethod
    def _polys(polys, poly_k):
        # the C ABI reads sum(2^k) words from the pointer it is given: check
        # the buffer holds them (a short device buffer would be read past)
        need = 4 * sum(1 << int(k) for k in poly_k if 0 <= int(k) <= 40)
        if isinstance(polys, DeviceArray):
            if polys.nbytes < need:
                raise WhirError(f"device polynomials hold {polys.nbytes} bytes, the layout needs {need}")
            return polys.ptr, 1, None
        if isinstance(polys, (list, tuple)):
            parts = [np.asarray(p, np.uint32) for p in polys]
            if len(parts) != len(poly_k) or any(q.size != 1 << int(k) for q, k in zip(parts, poly_k)):
                raise WhirError("each polynomial must hold 2^k words for its k")
            flat = np.ascontiguousarray(np.concatenate(parts), np.uint32)
        else:
            flat = np.ascontiguousarray(polys, np.uint32)
            if flat.nbytes < need:
                raise WhirError(f"polynomials hold {flat.nbytes} bytes, the layout needs {need}")
        return flat.ctypes.data, 0, flat

    def commit(self, transcript, polys, poly_k):
        ptr, dev, keep = self._polys(polys, poly_k)
        ks = (ctypes.c_int32 * len(poly_k))(*poly_k)
        _check(lib().whir_commit(self.h, transcript.h, ptr, dev, ks, len(poly_k)))

    def stack_eval(self, transcript, poly_id, point):
        pt, pp = _u32(point)
        out = np.empty(4, np.uint32)
        _check(lib().whir_stack_eval(self.h, transcript.h, poly_id, pp, out.ctypes.data_as(u32p)))
        return out

    def open(self, transcript):
        _check(lib().whir_open(self.h, transcript.h))

    def prove(self, transcript, polys, poly_k, groups):
        ptr, dev, keep = self._polys(polys, poly_k)
        ks = (ctypes.c_int32 * len(poly_k))(*poly_k)
        gn = (ctypes.c_int32 * max(1, len(groups)))(*[len(g) for g in groups])
        flat = [i for g in groups for i in g]
        gi = (ctypes.c_int32 * max(1, len(flat)))(*flat)
        _check(lib().whir_prove(self.h, transcript.h, ptr, dev, ks, len(poly_k), gn, len(groups),
                                gi))

    def close(self):
        if self.h:
            lib().whir_prover_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prove_harness(ctx, params, polys, poly_k, groups, whir=None):
    """Reference harness (crates/whir/src/test.rs:218-235): returns (proof, checkpoint)."""
    w = whir or Whir(ctx, *params)
    t = PoseidonWriter()
    w.prove(t, polys, poly_k, groups)
    cp = t.draw_base()
    return t.finalize(), cp


def fold_code_rounds(ctx, dev_codeword, k_data, folding, idx, scales, rs, r):
    """whir_fold_code_rounds: per round (c0, c2) of fold_with_code's pow claims
    (folding x 8 words) and the round-0 sum term (4 words)."""
    n = len(idx)
    ix = (ctypes.c_size_t * max(1, n))(*[int(i) for i in idx])
    sc, sp = _u32(scales)
    rsa, rsp = _u32(rs)
    ra, rp = _u32(r if len(r) else np.zeros(4, np.uint32))
    out = np.zeros(8 * folding + 4, np.uint32)
    _check(lib().whir_fold_code_rounds(ctx.h, dev_codeword.ptr, k_data, folding, ix, n, sp, rsp,
                                       rp, out.ctypes.data_as(u32p)))
    return out


DEBUG_CHECKS, DEBUG_NVTX, DEBUG_VERIFY_INLINE = 1, 2, 4


def debug_set(flags):
    """whir_debug_set: DEBUG_CHECKS (the reference's debug invariants),
    DEBUG_NVTX (NVTX ranges) and/or DEBUG_VERIFY_INLINE (verify hashes each
    opening where it reads it); 0 turns the debug mode off."""
    _check(lib().whir_debug_set(flags))


def batch_max(params):
    """The most polynomials one whir_prove_batch call takes for these parameters."""
    p = params if isinstance(params, Params) else Params(*params)
    out = ctypes.c_int32()
    _check(lib().whir_batch_max(ctypes.byref(p), ctypes.byref(out)))
    return out.value


def prove_batch(ctx, params, polys, claims=1, commit_only=False):
    """whir_prove_batch: the harness on each polynomial of one shape, in lock
    step.  polys: np.uint32 arrays of 2^k words, or DeviceArrays (all of one
    kind).  Returns [(proof bytes, checkpoint)] in input order."""
    p = params if isinstance(params, Params) else Params(*params)
    n = len(polys)
    on_device = n > 0 and isinstance(polys[0], DeviceArray)
    keep, ptrs = [], (vp * max(1, n))()
    for i, a in enumerate(polys):
        if on_device:
            if not isinstance(a, DeviceArray) or a.nbytes < 4 << p.k:
                raise WhirError("device polynomial smaller than 2^params.k words")
            ptrs[i] = a.ptr
        else:
            a = np.ascontiguousarray(a, np.uint32)
            if a.size != (1 << p.k):
                raise WhirError("polynomial size does not match params.k")
            keep.append(a)
            ptrs[i] = a.ctypes.data
    cap = 64 if commit_only else proof_bound(p, claims)
    buf = np.empty(cap * max(1, n), np.uint8)  # filled by the library up to each length
    lens = (ctypes.c_size_t * max(1, n))()
    cps = np.zeros(max(1, n), np.uint32)
    _check(lib().whir_prove_batch(ctx.h, ctypes.byref(p), ptrs, 1 if on_device else 0, n,
                                  0 if commit_only else claims, 1 if commit_only else 0,
                                  ctypes.cast(buf.ctypes.data, ctypes.c_char_p), cap, lens,
                                  cps.ctypes.data_as(u32p)))
    out = []
    for i in range(n):
        if lens[i] > cap:
            raise WhirError("proof longer than its buffer")
        out.append((buf[i * cap:i * cap + lens[i]].tobytes(), int(cps[i])))
    return out


class Job:
    """One proving job for prove_jobs: the harness on one polynomial.

    poly: np.uint32 array of 2^k words (host) or a DeviceArray; claims:
    number of evaluation claims at transcript-drawn points; commit_only:
    commitment alone.  After prove_jobs: proof (bytes), checkpoint, status,
    worker, start_s, done_s, latency_s (done - arrival).
    """

    def __init__(self, params, poly, claims=1, commit_only=False, arrival_s=0.0):
        self.params = params if isinstance(params, Params) else Params(*params)
        self.poly = poly
        self.claims = claims
        self.commit_only = commit_only
        self.arrival_s = arrival_s
        self.proof = None
        self.checkpoint = None
        self.status = None
        self.worker = None
        self.start_s = None
        self.done_s = None

    @property
    def latency_s(self):
        return None if self.done_s is None else self.done_s - self.arrival_s


def workspace_bytes(params):
    """Device bytes one worker holds while proving with these parameters."""
    p = params if isinstance(params, Params) else Params(*params)
    out = ctypes.c_uint64()
    _check(lib().whir_workspace_bytes(ctypes.byref(p), ctypes.byref(out)))
    return out.value


def proof_bound(params, claims):
    """An upper bound of the proof length in bytes (sizes the output buffers)."""
    p = params if isinstance(params, Params) else Params(*params)
    out = ctypes.c_uint64()
    _check(lib().whir_proof_bytes_max(ctypes.byref(p), claims, ctypes.byref(out)))
    return out.value


def _jobs_in(jobs):
    n = len(jobs)
    arr = (JobC * max(1, n))()
    bufs, keep = [], []
    for i, j in enumerate(jobs):
        c = arr[i]
        c.params = j.params
        if isinstance(j.poly, DeviceArray):
            if 0 <= j.params.k <= 40 and j.poly.nbytes < 4 << j.params.k:
                raise WhirError("device polynomial smaller than 2^params.k words")
            c.poly, c.poly_on_device = j.poly.ptr, 1
        else:
            a = np.ascontiguousarray(j.poly, np.uint32)
            if a.size != (1 << j.params.k):
                raise WhirError("polynomial size does not match params.k")
            keep.append(a)
            c.poly, c.poly_on_device = a.ctypes.data, 0
        c.n_claims = 0 if j.commit_only else j.claims
        c.commit_only = 1 if j.commit_only else 0
        c.arrival_s = j.arrival_s
        cap = 64 if j.commit_only else proof_bound(j.params, j.claims)
        b = ctypes.create_string_buffer(cap)
        bufs.append(b)
        c.proof = ctypes.cast(b, ctypes.c_void_p)
        c.proof_cap = cap
    return arr, bufs, keep


def _jobs_out(jobs, arr, bufs):
    for i, j in enumerate(jobs):
        c = arr[i]
        j.status = c.status
        j.worker = c.worker
        j.start_s, j.done_s = c.start_s, c.done_s
        j.checkpoint = c.checkpoint
        j.proof = None
        if c.status == 0:
            if c.proof_len > c.proof_cap:
                raise WhirError("proof longer than its buffer")
            j.proof = bufs[i].raw[:c.proof_len]


class Server:
    """whir_server: a persistent pool of GPU workers (streams, pinned staging
    and prover buffers stay allocated between runs)."""

    def __init__(self, workers=8, device=0, budget_bytes=150 << 30, lockstep=0):
        h = vp()
        _check(lib().whir_server_new(device, workers, budget_bytes, ctypes.byref(h)))
        self.h = h.value
        self.workers = workers
        if lockstep:
            self.set_lockstep(lockstep)

    def set_lockstep(self, max_group):
        """Most same-shape jobs proved together in lock step (1: none; 0: default)."""
        _check(lib().whir_server_set_lockstep(self.h, max_group))

    def run(self, jobs, serve=False):
        """Runs the jobs (serve=True: each released at its arrival_s); fills
        their results and returns (wall seconds, peak device bytes)."""
        arr, bufs, keep = _jobs_in(jobs)
        st = RunStatsC()
        _check(lib().whir_server_run(self.h, arr, len(jobs), 1 if serve else 0,
                                     ctypes.byref(st)))
        _jobs_out(jobs, arr, bufs)
        return st.seconds, st.peak_device_bytes

    def close(self):
        if self.h:
            lib().whir_server_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def prove_jobs(jobs, workers=4, device=0, budget_bytes=150 << 30, serve=False):
    """whir_batch_prove (serve=False: all jobs released at once) or whir_serve
    (jobs released at their arrival_s) on a temporary worker pool.  Fills each
    Job's results; returns (wall seconds, peak device bytes held)."""
    arr, bufs, keep = _jobs_in(jobs)
    st = RunStatsC()
    fn = lib().whir_serve if serve else lib().whir_batch_prove
    _check(fn(device, arr, len(jobs), workers, budget_bytes, ctypes.byref(st)))
    _jobs_out(jobs, arr, bufs)
    return st.seconds, st.peak_device_bytes


def serve_simulate(arrival_s, need_bytes, duration_s, workers, budget_bytes, shape=None,
                   max_group=1):
    """Admission order of whir_serve with host sleeps standing in for proofs:
    returns (start_s, done_s, worker, status) arrays.  With shape (one id per
    job), jobs of equal shape that have arrived are grouped, up to max_group
    (whir_serve_simulate_groups).  A negative duration injects a proof that
    fails after |duration| seconds (status WHIR_ERR_INTERNAL)."""
    n = len(arrival_s)
    A = (ctypes.c_double * max(1, n))(*arrival_s)
    N = (ctypes.c_uint64 * max(1, n))(*[int(x) for x in need_bytes])
    D = (ctypes.c_double * max(1, n))(*duration_s)
    S = (ctypes.c_double * max(1, n))()
    E = (ctypes.c_double * max(1, n))()
    Wk = np.zeros(max(1, n), np.int32)
    St = np.zeros(max(1, n), np.int32)
    if shape is None:
        _check(lib().whir_serve_simulate(A, N, D, n, workers, budget_bytes, S, E,
                                         Wk.ctypes.data_as(i32p), St.ctypes.data_as(i32p)))
    else:
        sh = np.ascontiguousarray(shape, np.int32)
        _check(lib().whir_serve_simulate_groups(A, N, D, sh.ctypes.data_as(i32p), max_group, n,
                                                workers, budget_bytes, S, E,
                                                Wk.ctypes.data_as(i32p), St.ctypes.data_as(i32p)))
    return np.array(S[:n]), np.array(E[:n]), Wk[:n], St[:n]


def verify(params, poly_k, groups, proof):
    """Whir::verify on the host: returns (result, checkpoint); result 0 means
    accepted (see whir_verify for the rejection codes)."""
    p = params if isinstance(params, Params) else Params(*params)
    ks = (ctypes.c_int32 * len(poly_k))(*poly_k)
    gn = (ctypes.c_int32 * max(1, len(groups)))(*[len(g) for g in groups])
    flat = [i for g in groups for i in g]
    gi = (ctypes.c_int32 * max(1, len(flat)))(*flat)
    res = ctypes.c_int32()
    cp = np.zeros(1, np.uint32)
    _check(lib().whir_verify(ctypes.byref(p), ks, len(poly_k), gn, len(groups), gi, bytes(proof),
                             len(proof), ctypes.byref(res), cp.ctypes.data_as(u32p)))
    return res.value, int(cp[0])


def verify_batch(ctx, params, poly_k, groups, proofs):
    """whir_verify_batch: every proof (bytes) checked against the same
    parameters, polynomial sizes and claim groups, the Merkle openings of all
    of them hashed in one GPU launch; returns [(result, checkpoint)] as
    verify() gives for each proof alone."""
    p = params if isinstance(params, Params) else Params(*params)
    ks = (ctypes.c_int32 * len(poly_k))(*poly_k)
    gn = (ctypes.c_int32 * max(1, len(groups)))(*[len(g) for g in groups])
    flat = [i for g in groups for i in g]
    gi = (ctypes.c_int32 * max(1, len(flat)))(*flat)
    n = len(proofs)
    bufs = [np.frombuffer(bytes(pr), np.uint8) if len(pr) else np.zeros(1, np.uint8)
            for pr in proofs]
    ptrs = (ctypes.c_void_p * max(1, n))(*[b.ctypes.data for b in bufs])
    lens = (ctypes.c_size_t * max(1, n))(*[len(pr) for pr in proofs])
    res = np.zeros(max(1, n), np.int32)
    cps = np.zeros(max(1, n), np.uint32)
    _check(lib().whir_verify_batch(ctx.h, ctypes.byref(p), ks, len(poly_k), gn, len(groups), gi,
                                   n, ptrs, lens, res.ctypes.data_as(i32p),
                                   cps.ctypes.data_as(u32p)))
    return [(int(res[i]), int(cps[i])) for i in range(n)]


def autotune(ctx, log_h_lo, log_h_hi):
    """Pick the fastest tree / DFT launch splits for these sizes (process-wide);
    returns the text report."""
    buf = ctypes.create_string_buffer(1 << 16)
    _check(lib().whir_autotune(ctx.h, log_h_lo, log_h_hi, buf, len(buf)))
    return buf.value.decode()


def tune_tree(log_h, wide_log, split):
    _check(lib().whir_tune_tree(log_h, wide_log, split))


def tune_dft(log_h, width, l1_bias):
    _check(lib().whir_tune_dft(log_h, width, l1_bias))


def tune_reset():
    _check(lib().whir_tune_reset())
