"""Writes tests/golden/config4_mcowner.npz: Monte-Carlo value labels for the
distillation configuration -- the reference's own Playout::mc_owner(state,
64) (Playout.cpp:174-217), run by oracle/_ref/ref_harness, on N seeded
positions (default 1,048,576).

    LEELA_REF=/path/to/reference python tests/golden/make_config4.py [--n N] [--threads T]

Positions: oracle.config_boards(N, seed=4) (empty board, k ~ U[0, 250]
uniform legal moves, simple ko), identical on every host, so only the labels
are stored: the win rate of the side to move over 64 playouts is a multiple
of 1/64 (a drawn playout counts 1/2, so of 1/128), kept exactly as uint8
(w * 128), with checksums of the boards they belong to.  The reference's
playouts draw from per-thread random streams seeded from the clock, so a
rerun gives other, equally valid, labels.

The harness runs with the reference's own thread pool; `--chunk` positions
go to it per call, so an interrupted run keeps the chunks already written
(`--resume`).
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

SEED = 4
PLAYOUTS = 64
OUT = os.path.join(HERE, "config4_mcowner.npz")


def board_checksums(sq, tm):
    return (hashlib.sha256(sq.tobytes()).hexdigest()[:16], hashlib.sha256(tm.tobytes()).hexdigest()[:16])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--chunk", type=int, default=65536)
    ap.add_argument("--ref", default=os.environ.get("LEELA_REF"))
    ap.add_argument("--work", default=None, help="directory for partial chunks (kept for --resume)")
    ap.add_argument("--resume", action="store_true")
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        ap.error("set LEELA_REF (or --ref) to the reference sources")
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "all", "ref", f"REF={args.ref}"],
                   check=True)
    harness = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    t0 = time.time()
    sq, tm, mv = O.config_boards(args.n, SEED)
    print(f"{args.n} positions generated in {time.time() - t0:.0f} s", flush=True)
    work = args.work or tempfile.mkdtemp(prefix="config4_")
    os.makedirs(work, exist_ok=True)
    labels = np.empty(args.n, np.uint8)
    for c0 in range(0, args.n, args.chunk):
        c1 = min(args.n, c0 + args.chunk)
        done = os.path.join(work, f"labels_{c0}.u8")
        if args.resume and os.path.exists(done):
            labels[c0:c1] = np.fromfile(done, np.uint8)
            continue
        pre = os.path.join(work, "chunk")
        np.ascontiguousarray(sq[c0:c1]).tofile(pre + ".sq")
        np.ascontiguousarray(tm[c0:c1]).tofile(pre + ".tm")
        np.ascontiguousarray(mv[c0:c1]).tofile(pre + ".mv")
        subprocess.run([harness, "mcfile", pre + ".sq", pre + ".tm", pre + ".mv", str(c1 - c0), str(PLAYOUTS),
                        str(args.threads), pre], check=True)
        w = np.fromfile(pre + ".mcowner", np.float32)
        x = np.rint(w * 128)
        assert np.allclose(x, w * 128, atol=1e-3) and x.min() >= 0 and x.max() <= 128
        labels[c0:c1] = x.astype(np.uint8)
        labels[c0:c1].tofile(done)
        print(f"{c1}/{args.n} labelled, {time.time() - t0:.0f} s", flush=True)
    s_sq, s_tm = board_checksums(sq, tm)
    np.savez_compressed(OUT, winrate_x128=labels, seed=np.int64(SEED), n=np.int64(args.n),
                        playouts=np.int64(PLAYOUTS), squares_sha256=s_sq, to_move_sha256=s_tm)
    print(f"wrote {OUT}: {args.n} labels, mean win rate {labels.mean() / 128:.4f}, "
          f"{time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main()
