"""Writes tests/golden/config2_f64.npz: the FP64 oracle's answers for the
65,536 positions of the precision-variant configuration (config 2).

    python tests/golden/make_config2.py [--threads N]

Positions: oracle.config_boards(65536, seed=2) -- from the empty board,
k ~ U[0, 250] uniform legal non-pass moves (simple ko, no suicide), one
splitmix64 stream per position, the same on every host (the file keeps a
checksum of the boards so that a test on another host can confirm it
regenerates them).  Input planes: planes 0..23 of the policy and value sets
(oracle.gather_planes, pinned bit-exact against the reference's gather).
Nets: the benchmark nets (5x5 24->128, 11x 3x3 128->128, 1x1 head, ReLU;
value FC 361->256 ReLU -> FC 256->1 -> tanh) with the He-normal weights of
seeds 1 (policy) and 2 (value).

Stored per position (FP64 arithmetic on the exact FP32 weights):
  top1, top2   the two largest policy logits' points (int16)
  gap          logit[top1] - logit[top2] (float32)
  value        the value net's output (float32)
and, for the first 8,192 positions, the policy top-1 of FP64 arithmetic on
weights rounded to BF16 (top1_w_bf16) and to FP16 (top1_w_fp16): the
agreement a 16-bit weight format allows before any activation is rounded.

Takes about 12 minutes on 8 x86 cores (OpenBLAS dgemm, one thread per
position).
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

N_POS = 65536
SEED = 2
N_CAP = 8192
CHUNK = 2048


def sha16(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--n", type=int, default=N_POS)
    args = ap.parse_args()
    n = args.n
    t0 = time.time()
    sq, tm, _ = O.config_boards(n, SEED)
    P, V = O.make_net(O.CFG_POLICY), O.make_net(O.CFG_VALUE)
    wp, wv = O.he_weights(P, O.POLICY_SEED), O.he_weights(V, O.VALUE_SEED)
    wp_b, wp_h = O.quantize_weights(P, wp, "bf16"), O.quantize_weights(P, wp, "fp16")
    top1 = np.empty(n, np.int16)
    top2 = np.empty(n, np.int16)
    gap = np.empty(n, np.float32)
    value = np.empty(n, np.float32)
    ncap = min(n, N_CAP)
    cap_b = np.empty(ncap, np.int16)
    cap_h = np.empty(ncap, np.int16)
    if not O.enable_blas():
        print("warning: no OpenBLAS, plain loops (slow)", flush=True)
    for c0 in range(0, n, CHUNK):
        c1 = min(n, c0 + CHUNK)
        pp = O.gather_planes(sq[c0:c1], tm[c0:c1], 0)
        pv = O.gather_planes(sq[c0:c1], tm[c0:c1], 1)
        lg = O.forward_f64(P, wp, pp, args.threads)
        order = np.argsort(-lg, axis=1, kind="stable")
        top1[c0:c1] = order[:, 0]
        top2[c0:c1] = order[:, 1]
        gap[c0:c1] = lg[np.arange(c1 - c0), order[:, 0]] - lg[np.arange(c1 - c0), order[:, 1]]
        value[c0:c1] = O.forward_f64(V, wv, pv, args.threads)
        if c0 < ncap:
            k1 = min(c1, ncap)
            cap_b[c0:k1] = O.forward_f64(P, wp_b, pp[:k1 - c0], args.threads).argmax(1)
            cap_h[c0:k1] = O.forward_f64(P, wp_h, pp[:k1 - c0], args.threads).argmax(1)
        print(f"{c1}/{n} positions, {time.time() - t0:.0f} s", flush=True)
    O.disable_blas()
    np.savez_compressed(os.path.join(HERE, "config2_f64.npz"), top1=top1, top2=top2, gap=gap, value=value,
                        top1_w_bf16=cap_b, top1_w_fp16=cap_h,
                        squares_sha256=np.str_(sha16(sq)), to_move_sha256=np.str_(sha16(tm)),
                        seed=np.int64(SEED), n=np.int64(n))
    print("done", time.time() - t0)


if __name__ == "__main__":
    main()
