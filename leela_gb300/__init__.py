"""leela_gb300 -- GB300-native evaluation of Leela's policy and value nets.

Python host mirror of the engine's Network interface (Network.h:23-88) over
the C ABI in include/leela_gpu.h (libleela_gb300.so, built in-tree from
leela_gb300/csrc by leela_gb300.build).  There is no CPU fallback: if the
library is missing or no GPU is present the calls raise.

    ctx = Context(policy=NetDesc.config1_policy(w_p, "bf16"),
                  value=NetDesc.config1_value(w_v, "bf16"), max_batch=256)
    probs = ctx.policy(planes)            # planes uint8 [B][c_in][361]
    values = ctx.value(planes_v)

Network-level helpers follow the reference:
  get_scored_moves()  gather planes -> rotate -> forward -> un-rotate -> keep
                      EMPTY points -> prune losing ladders (Network.cpp:624-674,
                      742-832)
  rotate_nn_idx / rev_rotate_nn_idx  (Network.cpp:1341-1379)
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libleela_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "leela_gpu.h")

POINTS = 361
LG_FP32, LG_BF16, LG_FP8W, LG_FP16 = 0, 1, 2, 3
LG_ACT_ELU, LG_ACT_RELU = 0, 1
LG_NET_POLICY, LG_NET_VALUE, LG_NET_POLICY_LOGITS = 0, 1, 2
(PROF_TC_3X3, PROF_TC_HEAD, PROF_TC_FIRST, PROF_FP32_CONV, PROF_OTHER, PROF_TC_TRUNK, PROF_PACK,
 PROF_TAIL, PROF_LAT) = range(9)
PRECISIONS = {"fp32": LG_FP32, "bf16": LG_BF16, "fp8w": LG_FP8W, "fp8": LG_FP8W, "fp16": LG_FP16}

ERRORS = {-1: "bad argument", -2: "allocation failed", -3: "CUDA error", -4: "timeout",
          -5: "device error status"}


class LeelaGPUError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)} ({code}): {msg}")
        self.code = code


class _Desc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "c_in", "width1", "width", "n3x3", "head_k", "act", "act_head", "value_head",
        "fc_hidden", "value_map", "precision")] + [("weights", ctypes.c_void_p)]


_lib = None
_lib_lock = threading.Lock()

EXPORTS = ["lg_weight_count", "lg_create", "lg_destroy", "lg_last_error", "lg_policy",
           "lg_value", "lg_policy_device", "lg_value_device", "lg_submit", "lg_poll",
           "lg_stats", "lg_device_error", "lg_inject_fault", "lg_inject_stall", "lg_profile", "lg_profile_read",
           "lg_policy_device_static", "lg_autotune", "lg_tuning", "lg_set_tuning",
           "lg_policy_avg8_device", "lg_value_avg8_device", "lg_weights_save",
           "lg_weights_load"]


def library():
    """Loads libleela_gb300.so (raises if it has not been built)."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise LeelaGPUError(-3, f"{LIB_PATH} not built; run leela_gb300.build.build()")
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.POINTER
            vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
            L.lg_weight_count.argtypes = [P(_Desc)]
            L.lg_weight_count.restype = ctypes.c_size_t
            L.lg_create.argtypes = [P(_Desc), P(_Desc), i32, i32, P(vp)]
            L.lg_destroy.argtypes = [vp]
            L.lg_destroy.restype = None
            L.lg_last_error.restype = ctypes.c_char_p
            L.lg_policy.argtypes = [vp, vp, i32, f32, vp, vp]
            L.lg_value.argtypes = [vp, vp, i32, vp]
            L.lg_policy_device.argtypes = [vp, vp, i32, f32, vp, vp, vp]
            L.lg_value_device.argtypes = [vp, vp, i32, vp, vp]
            L.lg_submit.argtypes = [vp, i32, vp, i32, f32, vp, vp]
            L.lg_poll.argtypes = [vp, P(vp), i32, i32]
            L.lg_stats.argtypes = [vp, P(ctypes.c_longlong), P(ctypes.c_longlong)]
            L.lg_inject_fault.argtypes = [vp, i32]
            L.lg_inject_stall.argtypes = [vp, i32, i32]
            L.lg_device_error.argtypes = [vp]
            L.lg_profile.argtypes = [vp, i32]
            L.lg_policy_device_static.argtypes = [vp, vp, i32, f32, vp, vp, vp]
            L.lg_autotune.argtypes = [vp, ctypes.c_char_p, i32]
            L.lg_tuning.argtypes = [vp, i32, P(i32), P(i32)]
            L.lg_set_tuning.argtypes = [vp, i32, i32, i32]
            L.lg_policy_avg8_device.argtypes = [vp, vp, i32, f32, vp, vp]
            L.lg_weights_save.argtypes = [ctypes.c_char_p, P(_Desc), P(ctypes.c_char_p), i32]
            L.lg_weights_load.argtypes = [ctypes.c_char_p, i32, P(_Desc), ctypes.c_char_p, vp,
                                          ctypes.c_size_t, P(ctypes.c_size_t)]
            L.lg_value_avg8_device.argtypes = [vp, vp, i32, vp, vp]
            L.lg_profile_read.argtypes = [vp, i32, P(ctypes.c_longlong), P(ctypes.c_double)]
            L.lg_gather_device.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp]
            L.lg_policy_boards.argtypes = [vp, vp, vp, vp, i32, f32, vp, vp]
            L.lg_value_boards.argtypes = [vp, vp, vp, vp, i32, vp]
            _lib = L
    return _lib


def _check(rc):
    if rc < 0:
        msg = library().lg_last_error()
        raise LeelaGPUError(rc, msg.decode() if msg else "")
    return rc


class NetDesc:
    """Shape + weights of one net (see lg_net_desc in include/leela_gpu.h)."""

    def __init__(self, weights, c_in, width1, width, n3x3, head_k, act, act_head, value_head,
                 fc_hidden=0, value_map=0, precision="fp32"):
        self.shape = dict(c_in=c_in, width1=width1, width=width, n3x3=n3x3, head_k=head_k,
                          act=act, act_head=act_head, value_head=value_head, fc_hidden=fc_hidden,
                          value_map=value_map)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else precision
        self.weights = np.ascontiguousarray(weights, dtype=np.float32)
        n = self.weight_count()
        if self.weights.size != n:
            raise ValueError(f"weights have {self.weights.size} floats, shape needs {n}")

    def _struct(self):
        return _Desc(precision=self.precision, weights=self.weights.ctypes.data, **self.shape)

    def weight_count(self):
        d = _Desc(precision=self.precision, weights=None, **self.shape)
        return int(library().lg_weight_count(ctypes.byref(d)))

    @property
    def c_in(self):
        return self.shape["c_in"]

    @property
    def value_head(self):
        return bool(self.shape["value_head"])

    # Benchmark nets: 5x5 24->128, 11x 3x3 128->128, 1x1 head, ReLU; value
    # FC 361->256 ReLU, FC 256->1, tanh.
    @classmethod
    def config1_policy(cls, w, precision="fp32"):
        return cls(w, 24, 128, 128, 11, 1, LG_ACT_RELU, 0, 0, precision=precision)

    @classmethod
    def config1_value(cls, w, precision="fp32"):
        return cls(w, 24, 128, 128, 11, 1, LG_ACT_RELU, 0, 1, 256, 0, precision=precision)

    # The reference's own BLAS-build shapes (Network.cpp:783-807, 709-737).
    @classmethod
    def reference_policy(cls, w, precision="fp32"):
        return cls(w, 32, 96, 128, 11, 3, LG_ACT_ELU, 1, 0, precision=precision)

    @classmethod
    def reference_value(cls, w, precision="fp32"):
        return cls(w, 32, 64, 64, 10, 3, LG_ACT_ELU, 1, 1, 256, 1, precision=precision)


class Context:
    """One GPU context holding a policy and/or a value net."""

    def __init__(self, policy: NetDesc | None = None, value: NetDesc | None = None,
                 device: int = 0, max_batch: int = 256):
        L = library()
        self._h = ctypes.c_void_p()
        self.policy_desc, self.value_desc = policy, value
        self.max_batch = max_batch
        ps = policy._struct() if policy else None
        vs = value._struct() if value else None
        _check(L.lg_create(ctypes.byref(ps) if ps else None, ctypes.byref(vs) if vs else None,
                           device, max_batch, ctypes.byref(self._h)))

    def close(self):
        if self._h:
            library().lg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- host-buffer calls (blocking)
    def policy(self, planes, temperature: float = 1.0, return_logits: bool = False):
        planes = np.ascontiguousarray(planes, dtype=np.uint8)
        B = planes.shape[0]
        probs = np.empty((B, POINTS), dtype=np.float32)
        logits = np.empty((B, POINTS), dtype=np.float32) if return_logits else None
        _check(library().lg_policy(self._h, planes.ctypes.data, B, temperature, probs.ctypes.data,
                                   logits.ctypes.data if logits is not None else None))
        return (probs, logits) if return_logits else probs

    def value(self, planes):
        planes = np.ascontiguousarray(planes, dtype=np.uint8)
        B = planes.shape[0]
        out = np.empty(B, dtype=np.float32)
        _check(library().lg_value(self._h, planes.ctypes.data, B, out.ctypes.data))
        return out

    def policy_boards(self, squares, to_move, temperature: float = 1.0,
                      return_logits: bool = False, moves=None):
        """lg_policy_boards: boards in (squares [B][361], 0 black / 1 white /
        2 empty; to_move [B]; moves [B][4] = last move, the move before it,
        ko point (-1 none), white-has-komi flag, needed by nets reading
        planes 24..31), input planes gathered on the GPU."""
        squares, to_move, moves = _boards(squares, to_move, moves)
        B = squares.shape[0]
        probs = np.empty((B, POINTS), dtype=np.float32)
        logits = np.empty((B, POINTS), dtype=np.float32) if return_logits else None
        _check(library().lg_policy_boards(self._h, squares.ctypes.data, to_move.ctypes.data,
                                          moves.ctypes.data if moves is not None else None, B,
                                          temperature, probs.ctypes.data,
                                          logits.ctypes.data if logits is not None else None))
        return (probs, logits) if return_logits else probs

    def value_boards(self, squares, to_move, moves=None):
        squares, to_move, moves = _boards(squares, to_move, moves)
        B = squares.shape[0]
        out = np.empty(B, dtype=np.float32)
        _check(library().lg_value_boards(self._h, squares.ctypes.data, to_move.ctypes.data,
                                         moves.ctypes.data if moves is not None else None, B,
                                         out.ctypes.data))
        return out

    # ---- device-pointer calls (non-blocking, on `stream`)
    def policy_device(self, planes_ptr: int, B: int, probs_ptr: int, temperature: float = 1.0,
                      logits_ptr: int | None = None, stream: int | None = None):
        _check(library().lg_policy_device(self._h, planes_ptr, B, temperature, probs_ptr,
                                          logits_ptr, stream))

    def policy_device_static(self, planes_ptr: int, B: int, probs_ptr: int,
                             temperature: float = 1.0, logits_ptr: int | None = None,
                             stream: int | None = None):
        """lg_policy_device_static: FP32 policy, B <= 4, scratch in the
        library's static device array (no allocation)."""
        _check(library().lg_policy_device_static(self._h, planes_ptr, B, temperature, probs_ptr,
                                                 logits_ptr, stream))

    def policy_avg8_device(self, planes_ptr: int, B: int, probs_ptr: int,
                           temperature: float = 1.0, stream: int | None = None):
        """AVERAGE_ALL: the 8 symmetries of each position in one batch,
        un-rotated and averaged on the device (board order)."""
        _check(library().lg_policy_avg8_device(self._h, planes_ptr, B, temperature, probs_ptr,
                                               stream))

    def value_avg8_device(self, planes_ptr: int, B: int, value_ptr: int,
                          stream: int | None = None):
        _check(library().lg_value_avg8_device(self._h, planes_ptr, B, value_ptr, stream))

    def value_device(self, planes_ptr: int, B: int, value_ptr: int, stream: int | None = None):
        _check(library().lg_value_device(self._h, planes_ptr, B, value_ptr, stream))

    # ---- batching server
    def submit(self, net: int, planes: np.ndarray, out: np.ndarray, tag: int,
               temperature: float = 1.0):
        _check(library().lg_submit(self._h, net, planes.ctypes.data, planes.shape[0], temperature,
                                   out.ctypes.data, tag))

    def poll(self, max_tags: int = 64, timeout_us: int = 0):
        arr = (ctypes.c_void_p * max_tags)()
        n = _check(library().lg_poll(self._h, arr, max_tags, timeout_us))
        return [arr[i] for i in range(n)]

    def stats(self):
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        _check(library().lg_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return {"kernel_launches": a.value, "batches": b.value}

    def profile(self, enable: bool = True):
        _check(library().lg_profile(self._h, 1 if enable else 0))

    def profile_read(self, kind: int):
        n, ms = ctypes.c_longlong(), ctypes.c_double()
        _check(library().lg_profile_read(self._h, kind, ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def autotune(self, cache_path: str | None = None, force: bool = False):
        """Pick the tensor-core kernel per batch bucket (see lg_autotune)."""
        _check(library().lg_autotune(self._h, cache_path.encode() if cache_path else None,
                                     1 if force else 0))

    def tuning(self, B: int):
        a, b = ctypes.c_int(), ctypes.c_int()
        tuned = _check(library().lg_tuning(self._h, B, ctypes.byref(a), ctypes.byref(b)))
        return {"tuned": bool(tuned), "conv3x3": a.value, "first": b.value}

    def set_tuning(self, B: int, conv3x3: int, first: int):
        _check(library().lg_set_tuning(self._h, B, conv3x3, first))

    def inject_fault(self, nth_call: int):
        _check(library().lg_inject_fault(self._h, nth_call))

    def device_error(self) -> int:
        """lg_device_error: after the streams of earlier device-pointer calls
        were synchronized, LG_OK (0) or LG_ERR_DEVICE (-5) if one of their
        kernels gave up a bounded wait; the error word is cleared."""
        return int(library().lg_device_error(self._h))

    def inject_stall(self, kind: int, polls: int = 0):
        """lg_inject_stall: the next trunk (kind 0) or small-batch (kind 1)
        launch waits for a flag nothing publishes, with short limits."""
        _check(library().lg_inject_stall(self._h, kind, polls))


# ------------------------------------------------------------------ symmetry

def rotate_nn_idx(vertex: int, symmetry: int) -> int:
    """Network.cpp:1360-1379: symmetries 4..7 transpose first; then identity,
    flip y, flip x, flip both."""
    x, y = vertex % 19, vertex // 19
    if symmetry >= 4:
        x, y = y, x
        symmetry -= 4
    nx = 18 - x if symmetry & 2 else x
    ny = 18 - y if symmetry & 1 else y
    return ny * 19 + nx


_INVERT = (0, 1, 2, 3, 4, 6, 5, 7)


def rev_rotate_nn_idx(vertex: int, symmetry: int) -> int:
    return rotate_nn_idx(vertex, _INVERT[symmetry])


ROTATE = np.array([[rotate_nn_idx(i, s) for i in range(POINTS)] for s in range(8)], dtype=np.int64)
REV_ROTATE = np.array([[rev_rotate_nn_idx(i, s) for i in range(POINTS)] for s in range(8)],
                      dtype=np.int64)


def _boards(squares, to_move, moves):
    squares = np.ascontiguousarray(squares, dtype=np.int8).reshape(-1, POINTS)
    B = squares.shape[0]
    to_move = np.ascontiguousarray(np.broadcast_to(np.asarray(to_move, dtype=np.int8), (B,)))
    if moves is not None:
        moves = np.ascontiguousarray(moves, dtype=np.int32).reshape(B, 4)
    return squares, to_move, moves


def gather_device(squares_ptr: int, to_move_ptr: int, B: int, which: int, nplanes: int,
                  planes_ptr: int, stream: int | None = None, moves_ptr: int | None = None):
    """lg_gather_device: input planes 0..nplanes-1 (<= 32) of the policy
    (which=0) or value (which=1) set from boards, device pointers, on
    `stream`; moves_ptr ([B][4] int32) is needed for planes 24..31."""
    _check(library().lg_gather_device(squares_ptr, to_move_ptr, moves_ptr, B, which, nplanes,
                                      planes_ptr, stream))


def rotate_planes(planes: np.ndarray, symmetry: int) -> np.ndarray:
    """planes[..., 361] -> out[..., i] = planes[..., rotate_nn_idx(i, sym)]
    (Network.cpp:765-773)."""
    return np.ascontiguousarray(planes[..., ROTATE[symmetry]])


def get_scored_moves(ctx: Context, planes32: np.ndarray, squares: np.ndarray,
                     ladder: np.ndarray, rotation: int = 0, temperature: float = 1.0):
    """One position through the GPU policy net, returned as the reference's
    Netresult: [(prob, point)] over EMPTY points in y-major scan order, with
    losing-ladder points set to 0 (Network.cpp:656-667, 820-829).  `point` is
    y*19+x; squares uses FastBoard's codes (EMPTY = 2)."""
    c_in = ctx.policy_desc.c_in
    x = rotate_planes(planes32[:c_in], rotation)[None]
    probs = ctx.policy(x, temperature)[0]
    out = []
    for idx in range(POINTS):
        if squares[idx] == 2:
            val = float(probs[REV_ROTATE[rotation][idx]])
            if ladder[idx]:
                val = 0.0
            out.append((val, idx))
    return out


# ------------------------------------------------------------------ weight files

def save_weights(path: str, nets):
    """nets: list of (name, NetDesc).  Writes the checksummed weight file of
    lg_weights_save."""
    arr = (_Desc * len(nets))(*[d._struct() for _, d in nets])
    names = (ctypes.c_char_p * len(nets))(*[n.encode()[:15] for n, _ in nets])
    _check(library().lg_weights_save(path.encode(), arr, names, len(nets)))


def load_weights(path: str):
    """Returns [(name, NetDesc)] from a file written by save_weights."""
    L = library()
    out = []
    i = 0
    while True:
        d = _Desc()
        name = ctypes.create_string_buffer(16)
        count = ctypes.c_size_t()
        n = _check(L.lg_weights_load(path.encode(), i, ctypes.byref(d), name, None, 0,
                                     ctypes.byref(count)))
        w = np.empty(count.value, dtype=np.float32)
        _check(L.lg_weights_load(path.encode(), i, ctypes.byref(d), name, w.ctypes.data, w.size,
                                 ctypes.byref(count)))
        out.append((name.value.decode(), NetDesc(w, d.c_in, d.width1, d.width, d.n3x3, d.head_k,
                                                 d.act, d.act_head, d.value_head, d.fc_hidden,
                                                 d.value_map, precision=d.precision)))
        i += 1
        if i >= n:
            return out
