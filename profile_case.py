"""A small, self-contained launch of the vgh kernel for profiling.

Builds one 64^3 x 1024-spline table (FP32, FP16 or I16 storage; 0.6-1.2 GB)
and one batch of 64 walkers (about 17.6k points, 0.7 GB of outputs), then
runs the evaluation `--launches` times and prints the CUDA-event time of each.
Everything it touches is a few GB, larger than L2, so DRAM counters of one
launch mean what they mean in the benchmark.

    python profile_case.py --storage f16 --launches 3
    python profile_case.py --storage f16 --det 2048  # fused determinant ratio
    python profile_case.py --storage f32 --complex 1 --splines 256 --points 32768 --sort 1
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--storage", default="f16", choices=["f32", "f16", "bf16", "i16", "f64"])
    ap.add_argument("--fp64-mode", type=int, default=0, help="f64 tables: 1 evaluates in double-float arithmetic")
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--splines", type=int, default=1024)
    ap.add_argument("--walkers", type=int, default=64)
    ap.add_argument("--points", type=int, default=0, help="> 0: this many points instead of walkers' batches")
    ap.add_argument("--complex", type=int, default=0, help="1: complex splines (c, or z with --storage f64)")
    ap.add_argument("--vgh", type=int, default=1)
    ap.add_argument("--tile", type=int, nargs=3, default=None)
    ap.add_argument("--sort", type=int, default=0)
    ap.add_argument("--mode", type=int, default=-1, help="load mode: 0 direct, 1 L2 prefetch, 2 smem pipeline, "
                    "3 wide smem pipeline (16-bit), 4 TMA pipeline, 5 tensor cores (F16, BF16)")
    ap.add_argument("--sweep", type=int, default=0, help="time every tile shape in every load mode")
    ap.add_argument("--det", type=int, default=0,
                    help="W > 0: time the fused determinant ratio (value, gradient, Laplacian; transposed "
                         "inverses) of W walkers over all splines instead")
    args = ap.parse_args()

    import torch
    from einspline_gb300 import api, synth
    st = {"f32": api.STORE_F32, "f16": api.STORE_F16, "bf16": api.STORE_BF16, "i16": api.STORE_I16,
          "f64": api.STORE_NATIVE}[args.storage]
    kind = ("z" if args.complex else "d") if args.storage == "f64" else ("c" if args.complex else "s")
    g = args.grid
    T = api.MultiUBspline3D(kind, [(0.0, 1.0, g)] * 3, [(api.PERIODIC, api.PERIODIC)] * 3, args.splines,
                            storage=st)
    cshape = (2,) if args.complex else ()
    buf = torch.empty((128, g, g, g) + cshape, dtype=torch.float64 if kind in "dz" else torch.float32, device="cuda")
    for f in range(0, args.splines, 128):
        n = min(128, args.splines - f)
        api.fill_uniform(buf[:n], 20261203, -1.0, 1.0, offset=f * g ** 3 * (2 if args.complex else 1))
        T.set_device(f, buf[:n])
    T.flush()
    del buf
    if kind in "dz":
        T.set_fp64_mode(args.fp64_mode)
    if args.det:
        # The ratio reads only row k of each transposed inverse: with k = 0 a
        # [W][1][N] buffer (row 0 of every walker's N x N matrix) is all the
        # kernel touches, so the capture holds megabytes, not W * N * N floats.
        W, N = args.det, args.splines
        Ai = torch.empty((W, 1, N), dtype=torch.float32, device="cuda")
        api.fill_uniform(Ai, 92, -1.0, 1.0)
        D = api.Determinants(Ai, Ai, N, trans=1)
        pos = torch.from_numpy(synth.points_uniform(779, W).astype(np.float32)).cuda()
        D.ratio(T, pos, 0, grad_lapl=True)
        torch.cuda.synchronize()
        times = []
        for _ in range(args.launches):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            D.ratio(T, pos, 0, grad_lapl=True)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        bpe = 64 * (4 if st == api.STORE_F32 else 2) + 4
        print(json.dumps({"storage": args.storage, "walkers": W, "orbitals": N, "ms": times, "bytes_per_eval": bpe,
                          "GBps": [W * N * bpe / (t * 1e-3) / 1e9 for t in times]}))
        return
    if args.tile:
        T.set_tile(*args.tile)
    T.set_load_mode(args.mode)
    npts = args.points if args.points > 0 else int(synth.walker_sizes(777, args.walkers).sum())
    pos = torch.from_numpy(synth.points_uniform(778, npts)).cuda()
    P = pos.shape[0]
    odt = torch.float64 if kind in "dz" else torch.float32
    ncol = args.splines * (2 if args.complex else 1)
    out = (torch.empty((P, ncol), dtype=odt, device="cuda"),
           torch.empty((P, ncol * 3), dtype=odt, device="cuda"),
           torch.empty((P, ncol * 6), dtype=odt, device="cuda"))
    torch.cuda.synchronize()
    if args.sweep:
        res = []
        for pf in (0, 1, 2, 3, 4):
            T.set_load_mode(pf)
            for tx in (32, 64, 128, 256):
                for ty in (1, 2, 4, 8):
                    if tx * ty > 256 or (pf >= 2 and ty > 1):
                        continue
                    for m in (1, 2, 4, 8):
                        pb = ty * m
                        T.set_tile(tx, ty, pb)
                        T.eval(pos, vgh=bool(args.vgh), rule=0, layout=0, sort=bool(args.sort), out=out)
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        e0.record()
                        for _ in range(3):
                            T.eval(pos, vgh=bool(args.vgh), rule=0, layout=0, sort=bool(args.sort), out=out)
                        e1.record()
                        torch.cuda.synchronize()
                        res.append((e0.elapsed_time(e1) / 3, pf, tx, ty, pb))
        res.sort()
        for r in res[:12]:
            print(json.dumps({"ms": r[0], "mode": r[1], "tile": r[2:]}))
        return
    times = []
    for _ in range(args.launches):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        T.eval(pos, vgh=bool(args.vgh), rule=0, layout=0, sort=bool(args.sort), out=out)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    if kind in "dc":
        bpe = 64 * 8 + (80 if args.vgh else 8)  # per (point, spline): 8-byte coefficients and outputs
    elif kind == "z":
        bpe = 64 * 16 + (160 if args.vgh else 16)
    else:
        bpe = 64 * (4 if st == api.STORE_F32 else 2) + (40 if args.vgh else 4)
    print(json.dumps({"storage": args.storage, "points": P, "splines": args.splines, "ms": times,
                      "tile": T.get_tile(), "bytes_per_eval": bpe,
                      "GBps": [P * args.splines * bpe / (t * 1e-3) / 1e9 for t in times]}))


if __name__ == "__main__":
    main()
