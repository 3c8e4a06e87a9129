"""Regenerates the golden fixtures in tests/golden from the reference engine.

Run where the reference sources (read-only) and g++ are present:

    LEELA_REF=/path/to/reference python tests/golden/make_golden.py [--only NAME ...]

(--ref overrides LEELA_REF; --only regenerates just the named fixtures,
e.g. --only config0, and leaves the others as they are.)

It builds oracle/_ref/ref_harness from the reference sources (oracle/Makefile
target `ref`) and the C restatement (oracle/liboracle.so), draws the
He-normal weights with the restatement's generator, and asks the reference's
own code for:

  positions_s0.npz     1024 seeded positions (empty board, komi 7.5, k~U[0,250]
                       uniform legal moves, seed 0): the 32 policy and 32 value
                       planes from the reference gather (Network.cpp:883-1201),
                       bit-packed; board squares; to-move/move number/k/ko point
                       (meta); last move, previous move, ko point as point
                       indices (-1 none) and the white-has-komi flag (moves)
  refexact_s0.npz      reference-shaped nets (Network.cpp:783-807, 709-737;
                       ELU, 3x3 heads): get_scored_moves(DIRECT, rot) probs
                       scattered to board order, the raw head output of the
                       convolve<> chain, get_value_internal(rot); 64 positions,
                       rotations 0 and 5
  config1_s0.npz       benchmark-shaped nets (5x5 24->128, 11x 3x3, 1x1 head,
                       ReLU, FC 361->256->1 tanh) through the reference's
                       im2col<> + cblas_sgemm + softmax: logits, probs, value;
                       64 positions, rotations 0 and 3
  config0_s0.npz       the same nets at DIRECT (rotation 0) for all 1024
                       positions: policy logits and values (the probabilities
                       follow from the logits by the reference softmax)
  weights.json         FNV-1a checksums of every weight set, so a test can
                       confirm another host draws the same weights
  mcowner_s0.npz       Playout::mc_owner(state, 64) for all 1024 positions (the
                       win rate of the side to move; the distilled net's value
                       labels).  The reference's playouts draw from per-thread
                       random streams, so a rerun with another thread schedule
                       gives other (equally valid) labels; the committed file
                       is the one the distillation tests were calibrated on.

The fixtures need nothing from the reference at test time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

N_POS = 1024
N_OUT = 64
SEED = 0


def run(cmd, env=None):
    print("+", " ".join(cmd), flush=True)
    subprocess.run(cmd, check=True, env=env)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("LEELA_REF"))
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--only", nargs="*", default=None,
                    choices=["positions", "refexact", "config1", "config0", "mcowner", "weights"])
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        ap.error("set LEELA_REF (or --ref) to the reference sources")
    want = (lambda name: True) if not args.only else (lambda name: name in args.only)

    odir = os.path.join(ROOT, "oracle")
    run(["make", "-s", "-C", odir, "liboracle.so"])
    run(["make", "-s", "-j8", "-C", odir, "ref", f"REF={args.ref}"])
    harness = os.path.join(odir, "_ref", "ref_harness")

    ref_p = O.make_net(O.REF_POLICY)
    ref_v = O.make_net(O.REF_VALUE)
    cfg_p = O.make_net(O.CFG_POLICY)
    cfg_v = O.make_net(O.CFG_VALUE)
    w_ref_p = O.he_weights(ref_p, O.POLICY_SEED)
    w_ref_v = O.he_weights(ref_v, O.VALUE_SEED)
    w_cfg_p = O.he_weights(cfg_p, O.POLICY_SEED)
    w_cfg_v = O.he_weights(cfg_v, O.VALUE_SEED)

    with tempfile.TemporaryDirectory() as td:
        wref = os.path.join(td, "ref_weights.bin")
        np.concatenate([w_ref_p, w_ref_v]).astype(np.float32).tofile(wref)
        wp = os.path.join(td, "cfg_p.bin")
        wv = os.path.join(td, "cfg_v.bin")
        w_cfg_p.tofile(wp)
        w_cfg_v.tofile(wv)
        env = dict(os.environ, LEELA_REF_WEIGHTS=wref)

        if want("positions"):
            pre = os.path.join(td, "pos")
            run([harness, "gen", str(N_POS), str(SEED), pre])
            pp = np.fromfile(pre + ".planes_p", np.uint8).reshape(N_POS, 32, 361)
            pv = np.fromfile(pre + ".planes_v", np.uint8).reshape(N_POS, 32, 361)
            sq = np.fromfile(pre + ".squares", np.int8).reshape(N_POS, 361)
            meta = np.fromfile(pre + ".meta", np.int32).reshape(N_POS, 4)
            moves = np.fromfile(pre + ".moves", np.int32).reshape(N_POS, 4)
            np.savez_compressed(os.path.join(HERE, "positions_s0.npz"),
                                planes_p=np.packbits(pp, axis=-1), planes_v=np.packbits(pv, axis=-1),
                                squares=sq, meta=meta, moves=moves)

        run([harness, "elucheck", wp], env=env)

        if want("config0"):
            pre = os.path.join(td, "cfg0all")
            run([harness, "config", str(N_POS), str(SEED), "0", wp, wv, pre], env=env)
            v = np.fromfile(pre + ".value", np.float32).reshape(N_POS, 2)
            np.savez_compressed(os.path.join(HERE, "config0_s0.npz"),
                                logits_r0=np.fromfile(pre + ".logits", np.float32).reshape(N_POS, 361),
                                value_pre_r0=v[:, 0], value_r0=v[:, 1])

        out = {}
        for rot in (0, 5) if want("refexact") else ():
            pre = os.path.join(td, f"refx{rot}")
            run([harness, "refexact", str(N_OUT), str(SEED), str(rot), pre], env=env)
            out[f"probs_r{rot}"] = np.fromfile(pre + ".probs", np.float32).reshape(N_OUT, 361)
            out[f"logits_r{rot}"] = np.fromfile(pre + ".logits", np.float32).reshape(N_OUT, 361)
            out[f"value_r{rot}"] = np.fromfile(pre + ".value", np.float32)
        if out:
            np.savez_compressed(os.path.join(HERE, "refexact_s0.npz"), **out)

        out = {}
        for rot in (0, 3) if want("config1") else ():
            pre = os.path.join(td, f"cfg{rot}")
            run([harness, "config", str(N_OUT), str(SEED), str(rot), wp, wv, pre], env=env)
            out[f"logits_r{rot}"] = np.fromfile(pre + ".logits", np.float32).reshape(N_OUT, 361)
            out[f"probs_r{rot}"] = np.fromfile(pre + ".probs", np.float32).reshape(N_OUT, 361)
            v = np.fromfile(pre + ".value", np.float32).reshape(N_OUT, 2)
            out[f"value_pre_r{rot}"] = v[:, 0]
            out[f"value_r{rot}"] = v[:, 1]
        if out:
            np.savez_compressed(os.path.join(HERE, "config1_s0.npz"), **out)

        if want("mcowner"):
            pre = os.path.join(td, "mc")
            run([harness, "mcowner", str(N_POS), str(SEED), "64", str(args.threads), pre])
            np.savez_compressed(os.path.join(HERE, "mcowner_s0.npz"),
                                mcowner=np.fromfile(pre + ".mcowner", np.float32))
        if not want("weights"):
            print("done")
            return

    sums = {
        "ref_policy": O.checksum(w_ref_p), "ref_value": O.checksum(w_ref_v),
        "cfg_policy": O.checksum(w_cfg_p), "cfg_value": O.checksum(w_cfg_v),
        "policy_seed": O.POLICY_SEED, "value_seed": O.VALUE_SEED,
        "first_weights_cfg_policy": [float(x) for x in w_cfg_p[:4]],
    }
    with open(os.path.join(HERE, "weights.json"), "w") as f:
        json.dump(sums, f, indent=1)
    print("done")


if __name__ == "__main__":
    main()
