"""Runs one frame pair of a workload preset through the stage API, for
profilers (ncu launch lists and single-kernel captures).

    python -m xbach.profile_frame [--preset 2] [--mode mixed|plain] [--runs 1]
                                  [--rank 0|1] [--rank-tau 0.3]

The pair is the preset's seeded synthetic pair (frame 0), device-resident;
each run is init (mask) -> sss -> cmv -> cd -> ksc -> conv -> sub on one
context, synchronised, and prints the kernel launches it made.  With
--rank 1 (mixed mode) the shipped ranker weights order the substamps, as in
the benchmark.  The first run of a context also times the autotuner's
variants, so launch lists are taken from the second run.
"""
import argparse
import pathlib
import sys


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--preset", type=int, default=2, choices=[1, 2, 3])
    ap.add_argument("--mode", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--rank", type=int, default=1)
    ap.add_argument("--rank-tau", type=float, default=0.3)
    args = ap.parse_args(argv)
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent.parent))
    import torch
    import xbach
    from xbach import ranker
    from xbach.synth import PARAMS_3, make_pair
    T, S, info = make_pair(args.preset)
    kw = dict(stampsx=info["stamps"], stampsy=info["stamps"], threshHigh=info["threshHigh"])
    if args.preset == 3:
        kw.update(PARAMS_3)
    mode = xbach.XB_MODE_PLAIN if args.mode == "plain" else xbach.XB_MODE_MIXED
    ctx = xbach.Context(xbach.default_params(mode=mode, **kw))
    if args.rank and mode == xbach.XB_MODE_MIXED:
        ranker.enable(ctx, ranker.preset5_weights(), policy=1, tau=args.rank_tau)
    dT = torch.from_numpy(T).cuda()
    dS = torch.from_numpy(S).cuda()
    h, w = T.shape
    for i in range(args.runs):
        l0 = ctx.launches()
        ctx.init_device(dT.data_ptr(), dS.data_ptr(), w, h)
        for stage in (ctx.sss, ctx.cmv, ctx.cd, ctx.ksc, ctx.conv, ctx.sub):
            stage()
        torch.cuda.synchronize()
        print(f"run {i}: {ctx.launches() - l0} kernel launches", flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
