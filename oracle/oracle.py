"""ctypes front end of the CPU oracle (leela_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product (leela_gb300) never
imports it.

Net presets follow the reference's shapes (Network.cpp:54-137, 783-807,
709-737) and the benchmark configurations (5x5 C_in->128, 11x 3x3 128->128,
1x1 head, ReLU, tanh value).
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

POINTS = 361


class OrNet(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "c_in", "width1", "width", "n3x3", "head_k", "act", "act_head",
        "value_head", "fc_hidden", "value_map")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def net(c_in, width1, width, n3x3, head_k, act, act_head, value_head, fc_hidden=0,
        value_map=0) -> OrNet:
    return OrNet(c_in, width1, width, n3x3, head_k, act, act_head, value_head, fc_hidden,
                 value_map)


ELU, RELU = 0, 1

# The reference's BLAS-build nets (Network.cpp:783-807, 709-737): ELU after
# every conv including the 3x3 head, value (1+tanh)/2.
REF_POLICY = dict(c_in=32, width1=96, width=128, n3x3=11, head_k=3, act=ELU, act_head=1,
                  value_head=0)
REF_VALUE = dict(c_in=32, width1=64, width=64, n3x3=10, head_k=3, act=ELU, act_head=1,
                 value_head=1, fc_hidden=256, value_map=1)
# Benchmark nets: 5x5 24->128, 11x 3x3 128->128, 1x1 128->1, ReLU after
# every conv but the last; value FC 361->256 ReLU, FC 256->1, tanh.
CFG_POLICY = dict(c_in=24, width1=128, width=128, n3x3=11, head_k=1, act=RELU, act_head=0,
                  value_head=0)
CFG_VALUE = dict(c_in=24, width1=128, width=128, n3x3=11, head_k=1, act=RELU, act_head=0,
                 value_head=1, fc_hidden=256, value_map=0)

POLICY_SEED = 1
VALUE_SEED = 2

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "leela_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.POINTER
            L.or_weight_count.argtypes = [P(OrNet)]
            L.or_weight_count.restype = ctypes.c_size_t
            L.or_conv_weight_offset.argtypes = [P(OrNet), ctypes.c_int]
            L.or_conv_weight_offset.restype = ctypes.c_size_t
            L.or_fc_weight_offset.argtypes = [P(OrNet)]
            L.or_fc_weight_offset.restype = ctypes.c_size_t
            L.or_n_conv.argtypes = [P(OrNet)]
            L.or_conv_shape.argtypes = [P(OrNet), ctypes.c_int] + [P(ctypes.c_int)] * 3
            L.or_he_weights.argtypes = [P(OrNet), ctypes.c_uint64, ctypes.c_void_p]
            L.or_checksum_f32.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
            L.or_checksum_f32.restype = ctypes.c_uint64
            L.or_forward_f32.argtypes = [P(OrNet), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
            L.or_forward_f64.argtypes = [P(OrNet), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p]
            for f in (L.or_forward_batch_f32, L.or_forward_batch_f64):
                f.argtypes = [P(OrNet), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                              ctypes.c_void_p, ctypes.c_int]
            L.or_softmax_f32.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                         ctypes.c_void_p]
            L.or_softmax_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_void_p]
            L.or_rotate_nn_idx.argtypes = [ctypes.c_int, ctypes.c_int]
            L.or_rev_rotate_nn_idx.argtypes = [ctypes.c_int, ctypes.c_int]
            L.or_rotate_planes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p]
            L.or_e4m3_round.argtypes = [ctypes.c_float]
            L.or_e4m3_round.restype = ctypes.c_float
            L.or_bf16_round.argtypes = [ctypes.c_float]
            L.or_bf16_round.restype = ctypes.c_float
            L.or_fp8_dequant_conv.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p]
            L.or_det_log.argtypes = [ctypes.c_double]
            L.or_det_log.restype = ctypes.c_double
            L.or_set_blas.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.or_time_pair_f32.argtypes = [P(OrNet), ctypes.c_void_p, P(OrNet), ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int]
            L.or_time_pair_f32.restype = ctypes.c_double
            L.or_gather_planes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_void_p]
            L.or_random_board.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p]
            L.or_config_board.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
            L.or_config_boards.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.or_config_boards.restype = None
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def make_net(preset: dict) -> OrNet:
    return net(**preset)


def weight_count(n: OrNet) -> int:
    return int(lib().or_weight_count(ctypes.byref(n)))


def he_weights(n: OrNet, seed: int) -> np.ndarray:
    w = np.empty(weight_count(n), dtype=np.float32)
    lib().or_he_weights(ctypes.byref(n), ctypes.c_uint64(seed), _ptr(w))
    return w


def checksum(w: np.ndarray) -> int:
    w = np.ascontiguousarray(w, dtype=np.float32)
    return int(lib().or_checksum_f32(_ptr(w), w.size))


def conv_shapes(n: OrNet):
    L = lib()
    out = []
    for l in range(L.or_n_conv(ctypes.byref(n))):
        k, ci, co = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.or_conv_shape(ctypes.byref(n), l, ctypes.byref(k), ctypes.byref(ci), ctypes.byref(co))
        out.append((k.value, ci.value, co.value,
                    int(L.or_conv_weight_offset(ctypes.byref(n), l))))
    return out


def forward_f32(n: OrNet, w: np.ndarray, planes: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """planes [B][c_in][361] uint8 -> [B][361] logits or [B] values (float32)."""
    planes = np.ascontiguousarray(planes, dtype=np.uint8).reshape(-1, n.c_in * POINTS)
    B = planes.shape[0]
    out = np.empty((B, 1 if n.value_head else POINTS), dtype=np.float32)
    rc = lib().or_forward_batch_f32(ctypes.byref(n), _ptr(w), _ptr(planes), B, _ptr(out), nthreads)
    if rc:
        raise RuntimeError("oracle forward failed")
    return out[:, 0] if n.value_head else out


def forward_f64(n: OrNet, w: np.ndarray, planes: np.ndarray, nthreads: int = 0) -> np.ndarray:
    planes = np.ascontiguousarray(planes, dtype=np.uint8).reshape(-1, n.c_in * POINTS)
    B = planes.shape[0]
    out = np.empty((B, 1 if n.value_head else POINTS), dtype=np.float64)
    rc = lib().or_forward_batch_f64(ctypes.byref(n), _ptr(w), _ptr(planes), B, _ptr(out), nthreads)
    if rc:
        raise RuntimeError("oracle forward failed")
    return out[:, 0] if n.value_head else out


def forward_layers_f32(n: OrNet, w: np.ndarray, planes: np.ndarray):
    """One position; returns (out, [per-layer activations [cout][361]])."""
    planes = np.ascontiguousarray(planes, dtype=np.uint8).reshape(n.c_in * POINTS)
    shapes = conv_shapes(n)
    acts = np.empty(sum(co for _, _, co, _ in shapes) * POINTS, dtype=np.float32)
    out = np.empty(POINTS, dtype=np.float32)
    rc = lib().or_forward_f32(ctypes.byref(n), _ptr(w), _ptr(planes), _ptr(out), _ptr(acts))
    if rc:
        raise RuntimeError("oracle forward failed")
    layers, off = [], 0
    for _, _, co, _ in shapes:
        layers.append(acts[off:off + co * POINTS].reshape(co, POINTS))
        off += co * POINTS
    return (out[0] if n.value_head else out), layers


def softmax_f32(x: np.ndarray, temperature: float = 1.0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    L = lib()
    for i in range(x.shape[0]) if x.ndim == 2 else [None]:
        xi = x[i] if i is not None else x
        oi = out[i] if i is not None else out
        L.or_softmax_f32(_ptr(xi), xi.size, ctypes.c_float(temperature), _ptr(oi))
    return out


def softmax_f64(x: np.ndarray, temperature: float = 1.0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    L = lib()
    for i in range(x.shape[0]) if x.ndim == 2 else [None]:
        xi = x[i] if i is not None else x
        oi = out[i] if i is not None else out
        L.or_softmax_f64(_ptr(xi), xi.size, ctypes.c_double(temperature), _ptr(oi))
    return out


def rotate_nn_idx(v: int, sym: int) -> int:
    return int(lib().or_rotate_nn_idx(v, sym))


def rev_rotate_nn_idx(v: int, sym: int) -> int:
    return int(lib().or_rev_rotate_nn_idx(v, sym))


def rotate_planes(planes: np.ndarray, sym: int) -> np.ndarray:
    planes = np.ascontiguousarray(planes, dtype=np.uint8)
    c = planes.size // POINTS
    out = np.empty_like(planes)
    lib().or_rotate_planes(_ptr(planes), c, sym, _ptr(out))
    return out


def gather_planes(squares: np.ndarray, to_move, which: int, nplanes: int = 24,
                  moves: np.ndarray | None = None) -> np.ndarray:
    """Planes 0..nplanes-1 (nplanes <= 32) of the policy (which=0) or value
    (which=1) input set for boards squares [B][361] (0 black, 1 white,
    2 empty) -> [B][nplanes][361] u8.  moves [B][4] (last move, the move
    before it, ko point, white-has-komi flag; point indices, -1 none) is
    needed for planes 24..31.  Restates Network::gather_features_policy /
    gather_features_value (Network.cpp:883-1201)."""
    sq = np.ascontiguousarray(squares, dtype=np.int8).reshape(-1, POINTS)
    tm = np.broadcast_to(np.asarray(to_move, dtype=np.int64), (sq.shape[0],))
    mv = None if moves is None else np.ascontiguousarray(moves, dtype=np.int32).reshape(-1, 4)
    out = np.empty((sq.shape[0], nplanes, POINTS), dtype=np.uint8)
    L = lib()
    for b in range(sq.shape[0]):
        L.or_gather_planes(_ptr(sq[b]), int(tm[b]), None if mv is None else _ptr(mv[b]), which, nplanes,
                           _ptr(out[b]))
    return out


def random_boards(n: int, seed: int, kmax: int = 300):
    """n boards after k ~ U[0, kmax] random legal moves (captures applied):
    (squares [n][361] int8, to_move [n] int8)."""
    rng = np.random.default_rng(seed)
    ks = rng.integers(0, kmax + 1, size=n)
    sq = np.empty((n, POINTS), dtype=np.int8)
    tm = np.empty(n, dtype=np.int8)
    L = lib()
    for i in range(n):
        tm[i] = L.or_random_board(seed * 1000003 + i, int(ks[i]), _ptr(sq[i]))
    return sq, tm


def config_boards(n: int, seed: int, kmax: int = 250, start: int = 0, threads: int | None = None):
    """Positions n of the benchmark configurations' kind (empty board,
    k ~ U[0, kmax] uniform legal moves, simple ko, no suicide), position i
    drawn from stream seed * 2**32 + start + i: (squares [n][361] int8,
    to_move [n] int8, moves [n][4] int32 = last move, the move before it,
    ko point, white-has-komi flag).  Large sets are generated in chunks on
    `threads` host threads (the C generator runs without the GIL); every
    position depends only on its own stream, so the result does not depend
    on the thread count."""
    sq = np.empty((n, POINTS), dtype=np.int8)
    tm = np.empty(n, dtype=np.int8)
    mv = np.empty((n, 4), dtype=np.int32)
    L = lib()
    base = ctypes.c_uint64(seed << 32)
    chunk = 4096

    def run(c0):
        c1 = min(n, c0 + chunk)
        L.or_config_boards(base, start + c0, c1 - c0, kmax, _ptr(sq[c0:]), _ptr(mv[c0:]), _ptr(tm[c0:]))

    starts = range(0, n, chunk)
    nt = threads or min(16, os.cpu_count() or 1)
    if n <= chunk or nt <= 1:
        for c0 in starts:
            run(c0)
    else:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(nt) as ex:
            list(ex.map(run, starts))
    return sq, tm, mv


def e4m3_round(x: float) -> float:
    return float(lib().or_e4m3_round(ctypes.c_float(x)))


def bf16_round_array(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    r = np.where(nan, u.astype(np.uint32), r)
    return r.view(np.float32).reshape(np.shape(x))


def fp16_round_array(x: np.ndarray) -> np.ndarray:
    """IEEE half, round to nearest even (as __float2half_rn), back to float32."""
    return np.asarray(x, dtype=np.float32).astype(np.float16).astype(np.float32)


def quantize_weights(n: OrNet, w: np.ndarray, mode: str) -> np.ndarray:
    """Weights as the low-precision paths see them: 'bf16' rounds every
    weight to BF16, 'fp16' to IEEE half (round to nearest even); 'fp8'
    quantises each conv's W per output channel to E4M3 (scale = max|w|/448)
    and keeps the dequantised values (FC layers stay BF16).  Biases stay
    FP32 in all three."""
    w = np.array(w, dtype=np.float32, copy=True)
    L = lib()
    rnd = fp16_round_array if mode == "fp16" else bf16_round_array
    for k, ci, co, off in conv_shapes(n):
        nw = co * ci * k * k
        W = np.ascontiguousarray(w[off:off + nw])
        if mode == "fp8":
            wq = np.empty_like(W)
            sc = np.empty(co, dtype=np.float32)
            L.or_fp8_dequant_conv(_ptr(W), co, ci * k * k, _ptr(wq), _ptr(sc))
            w[off:off + nw] = wq
        else:
            w[off:off + nw] = rnd(W)
    if n.value_head:
        off = int(L.or_fc_weight_offset(ctypes.byref(n)))
        h = n.fc_hidden
        w[off:off + h * POINTS] = rnd(w[off:off + h * POINTS])
        o2 = off + h * POINTS + h
        w[o2:o2 + h] = rnd(w[o2:o2 + h])
    return w


def find_openblas():
    """Path of the OpenBLAS that scipy bundles (LP64 'scipy_' symbols), or None."""
    try:
        import scipy
    except ImportError:
        return None
    d = os.path.dirname(scipy.__file__) + ".libs"
    c = sorted(glob.glob(os.path.join(d, "libscipy_openblas-*.so")))
    return c[0] if c else None


_blas = None


def enable_blas() -> bool:
    """Route the oracle's per-layer GEMM through OpenBLAS sgemm/dgemm, one
    BLAS thread per call, as the reference's BLAS build does
    (Network.cpp:239, 375-380)."""
    global _blas
    path = find_openblas()
    if not path:
        return False
    if _blas is None:
        _blas = ctypes.CDLL(path)
        _blas.scipy_openblas_set_num_threads(1)
    lib().or_set_blas(ctypes.cast(_blas.scipy_cblas_sgemm, ctypes.c_void_p),
                      ctypes.cast(_blas.scipy_cblas_dgemm, ctypes.c_void_p))
    return True


def disable_blas():
    lib().or_set_blas(None, None)


def time_pair_f32(pol: OrNet, wp, val: OrNet, wv, planes_p, planes_v, iters: int,
                  nthreads: int) -> float:
    planes_p = np.ascontiguousarray(planes_p, dtype=np.uint8)
    planes_v = np.ascontiguousarray(planes_v, dtype=np.uint8)
    npos = planes_p.shape[0]
    return float(lib().or_time_pair_f32(ctypes.byref(pol), _ptr(wp), ctypes.byref(val), _ptr(wv),
                                        _ptr(planes_p), _ptr(planes_v), npos, iters, nthreads))
