"""Command-line driver for the contraction-only path and the synthetic workloads.

    python -m hybridhsdla_gb300.driver contract data.in data.out [--precision ozaki|fp64] [--slices N]
        reads the reference's data.in (h_and_s.cpp:763-786), computes H and S on the GPU through
        hsdla_contract_ab, writes data.out (h_and_s.cpp:870-873) and prints the timing;
    python -m hybridhsdla_gb300.driver dump CONFIG DIR [--kpoints N]
        writes DIR/data.in for the first k-point of a synthetic configuration (the
        DUMP_FLAPW_DATA side of the reference, h_and_s.cpp:744-790);
    python -m hybridhsdla_gb300.driver run CONFIG [--kpoints N] [--precision ...]
        H and S of every k-point through hsdla_create_hs with per-k-point timings, in the
        spirit of the reference's h_and_s [dump_dir] [k_ind_max] (h_and_s.cpp:897-954).
"""
from __future__ import annotations

import argparse
import json
import os
import sys


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="hybridhsdla_gb300.driver")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("contract")
    c.add_argument("data_in")
    c.add_argument("data_out")
    c.add_argument("--precision", default="ozaki", choices=["ozaki", "fp64"])
    c.add_argument("--slices", type=int, default=0)
    d = sub.add_parser("dump")
    d.add_argument("config")
    d.add_argument("dir")
    r = sub.add_parser("run")
    r.add_argument("config")
    r.add_argument("--kpoints", type=int, default=0)
    r.add_argument("--precision", default="ozaki", choices=["ozaki", "fp64"])
    args = ap.parse_args(argv)

    from . import api, flapw_data, synth
    if args.cmd == "dump":
        s = synth.make_system(args.config)
        kp = s.kpoints[0]
        ctx = api.Context()
        pl = ctx.plan(s, kpoints=[kp])
        import numpy as np
        C = pl.construct_ab(0).cpu().numpy()
        A, B = api.split_ab(C, s.L, s.num_atoms)
        os.makedirs(args.dir, exist_ok=True)
        flapw_data.write_data_in(os.path.join(args.dir, "data.in"),
                                 flapw_data.from_system(s, kp, A, B, api.prepare_tmats(s)))
        print(json.dumps({"written": os.path.join(args.dir, "data.in"), "L": s.L, "a": s.num_atoms, "G": kp.n_g}))
        return 0
    if args.cmd == "contract":
        din = flapw_data.read_data_in(args.data_in)
        ctx = api.Context()
        H, S, rep = ctx.contract_ab(din, precision=args.precision, num_slices=args.slices)
        flapw_data.write_data_out(args.data_out, H, S)
        print(json.dumps({"G": din.G, "ms": rep["ms_total"], "tflops": rep["eff_tflops"],
                          "num_slices": rep["num_slices"]}))
        return 0
    if args.cmd == "run":
        s = synth.make_system(args.config)
        kps = s.kpoints[:args.kpoints] if args.kpoints else s.kpoints
        ctx = api.Context()
        tm = api.prepare_tmats(s)
        for i, kp in enumerate(kps):
            _, rep = ctx.create_hs(s, kpoints=[kp], precision=args.precision, tmats=tm)
            print(json.dumps({"k": i, "n_g": kp.n_g, "ms": rep["ms_total"], "tflops": rep["eff_tflops"]}))
        return 0
    return 2


if __name__ == "__main__":
    sys.exit(main())
