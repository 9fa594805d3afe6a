"""Command-line driver: the reference's ``h_and_s`` program and its data-file tools.

    python -m hybridhsdla_gb300.driver run DUMP [k_ind_max] [compute|store] [--precision ozaki|fp64]
                                           [--time-info PATH] [--batched]
        the reference's ``h_and_s [dump_dir] [k_ind_max] [compute|store]`` (``main`` and
        ``generate_matrices``, ``flapw_opt/src/h_and_s.cpp:897-954``): reads the Fleur dump
        (a directory holding fleur_dump.h5, the .h5 itself, or an .npz of the same quantities),
        builds the AtomData (radial solutions, T blocks), generates H and S for the first
        min(k_ind_max, k-points in the dump) k-points one create_HS2 call at a time (one
        hsdla_create_hs call each; --batched: all in one call) and saves the milliseconds per
        k-point to time.info in Armadillo's arma_ascii text format, as the reference does.
        The method argument is accepted and, as in the reference's STRIPPED build, ignored.
        DUMP may also name a synthetic configuration (hybridhsdla_gb300/synth.py).  When the
        dump carries Fleur's own H and S (the .npz fixture), their errors are printed too;
    python -m hybridhsdla_gb300.driver contract data.in data.out [--precision ozaki|fp64] [--slices N]
        reads the reference's data.in (h_and_s.cpp:763-786), computes H and S on the GPU through
        hsdla_contract_ab, writes data.out (h_and_s.cpp:870-873) and prints the timing;
    python -m hybridhsdla_gb300.driver dump CONFIG DIR
        writes DIR/data.in for the first k-point of a synthetic configuration (the
        DUMP_FLAPW_DATA side of the reference, h_and_s.cpp:744-790).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np


def write_time_info(path: str, ms) -> None:
    """``arma::vec::save(path, arma::arma_ascii)``: a header line, the dimensions, one value a line."""
    with open(path, "w") as f:
        f.write("ARMA_MAT_TXT_FN008\n%d 1\n" % len(ms))
        for v in ms:
            f.write("  %.16e\n" % float(v))


def read_time_info(path: str) -> np.ndarray:
    with open(path) as f:
        lines = f.read().split("\n")
    assert lines[0].startswith("ARMA_MAT_TXT_FN008")
    n = int(lines[1].split()[0])
    return np.array([float(x) for x in lines[2:2 + n]])


def _lower_errors(X, R):
    Xl, Rl = np.tril(X), np.tril(R)
    d = Xl - Rl
    return float(np.linalg.norm(d) / np.linalg.norm(Rl)), float(np.abs(d).max() / np.abs(Rl).max())


def run(source: str, k_ind_max: int = 60, precision: str = "ozaki", time_info: str = "time.info",
        batched: bool = False, out=sys.stdout):
    """h_and_s on a Fleur dump or a synthetic configuration; returns (per-k-point ms, results)."""
    from . import api, fleur_dump, synth
    golden = None
    if os.path.exists(source):
        d = fleur_dump.load(source)
        s = fleur_dump.to_system(d)
        if d.H_fleur is not None:
            golden = (d.H_fleur, d.S_fleur)
    else:
        s = synth.make_system(source)
    kps = s.kpoints[:min(k_ind_max, len(s.kpoints))]
    ctx = api.Context()
    tm = api.prepare_tmats(s)
    times, results = [], []
    if batched:
        res, rep = ctx.create_hs(s, kpoints=kps, precision=precision, tmats=tm)
        times = [rep["ms_per_kpoint"]] * len(kps)
        results = res
        print(json.dumps({"kpoints": len(kps), "ms": rep["ms_total"], "tflops": rep["eff_tflops"],
                          "num_slices": rep["num_slices"], "row_sets": rep["num_row_sets"]}), file=out)
    else:
        for i, kp in enumerate(kps):
            res, rep = ctx.create_hs(s, kpoints=[kp], precision=precision, tmats=tm)
            times.append(rep["ms_total"])
            results.append(res[0])
            print(json.dumps({"k": i, "n_g": kp.n_g, "ms": rep["ms_total"], "tflops": rep["eff_tflops"],
                              "num_slices": rep["num_slices"], "row_sets": rep["num_row_sets"],
                              "rotation_classes": rep["rotation_classes"]}), file=out)
    if golden is not None:
        H, S = results[0]
        eH, eS = _lower_errors(H, golden[0]), _lower_errors(S, golden[1])
        print(json.dumps({"vs_fleur_k0": {"H_fro": eH[0], "H_max": eH[1], "S_fro": eS[0], "S_max": eS[1]}}), file=out)
    if time_info:
        write_time_info(time_info, times)
    ctx.close()
    return times, results


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
    r.add_argument("source", help="Fleur dump (directory, fleur_dump.h5 or .npz) or a synthetic configuration")
    r.add_argument("k_ind_max", nargs="?", type=int, default=60)
    r.add_argument("method", nargs="?", default="store", choices=["compute", "store"])
    r.add_argument("--precision", default="ozaki", choices=["ozaki", "fp64"])
    r.add_argument("--time-info", default="time.info")
    r.add_argument("--batched", action="store_true")
    args = ap.parse_args(argv)

    from . import api, flapw_data, synth
    if args.cmd == "dump":
        s = synth.make_system(args.config)
        kp = s.kpoints[0]
        ctx = api.Context()
        pl = ctx.plan(s, kpoints=[kp])
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
        run(args.source, args.k_ind_max, args.precision, args.time_info, args.batched)
        return 0
    return 2


if __name__ == "__main__":
    sys.exit(main())
