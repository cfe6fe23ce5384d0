"""Trains the substamp ranker shipped as ranker_preset5.npy.

    python -m xbach.train_ranker [--out PATH] [--fields 2800]

Training data: the plain ksc loop's accept/reject labels on seeded preset-5
fields (defects on the bright candidates: hot science columns, variable
companions) at 2048^2 with 30k sources and 10x10 stamps, i.e. the stamp
width (183 px) and source density of the 4096^2 preset-5 frames; fields
0..N-1, about 110 labelled candidates each (2800 fields: 304,200).
Training: 20 epochs of Adam (batch 512, lr 3e-3, class-balanced
cross-entropy) with the library's CUDA kernels, which compute with the
weights rounded to BF16; the file holds those BF16 values (as float32).
Fields are generated in a spawned process pool (before CUDA starts in this
process) and labelled on the GPU in order, so the result is the same on
every run on the same GPU model.
"""
import argparse
import concurrent.futures as cf
import multiprocessing as mp
import os
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
DEFAULT_OUT = HERE / "ranker_preset5.npy"


def training_field(frame):
    sys.path.insert(0, str(HERE.parent))
    from xbach.synth import make_pair
    return make_pair(5, frame=frame, size=2048, n_src=30000, stamps=10)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(DEFAULT_OUT))
    ap.add_argument("--fields", type=int, default=2800)
    ap.add_argument("--epochs", type=int, default=20)
    args = ap.parse_args(argv)
    ex = cf.ProcessPoolExecutor(min(12, os.cpu_count() or 1), mp_context=mp.get_context("spawn"))
    sys.path.insert(0, str(HERE.parent))
    import xbach
    from xbach import ranker
    stats, pix, labels = [], [], []
    t0 = time.time()
    for c0 in range(0, args.fields, 48):
        for T, S, info in ex.map(training_field, range(c0, min(args.fields, c0 + 48))):
            p = xbach.default_params(stampsx=info["stamps"], stampsy=info["stamps"],
                                     threshHigh=info["threshHigh"], mode=xbach.XB_MODE_MIXED)
            st, px, lab, _ = ranker.labelled_frame(T, S, p)
            stats.append(st)
            pix.append(px)
            labels.append(lab)
    ex.shutdown()
    st, px, y = np.concatenate(stats), np.concatenate(pix), np.concatenate(labels)
    print(f"{len(y)} labelled candidates, {1 - y.mean():.3f} rejected ({time.time() - t0:.0f} s)")
    w, hist = ranker.train(st, px, y, epochs=args.epochs, batch=512, lr=3e-3)
    print(f"loss {hist[0]:.4f} -> {hist[-1]:.4f}")
    # the BF16 values the network computes with (nearest, ties to even)
    u = w.astype(np.float32).view(np.uint32).astype(np.uint64)
    w = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32)
    np.save(args.out, w)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
