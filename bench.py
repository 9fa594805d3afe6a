"""Benchmark of the H/S generation path on GB300.

One step = H and S (lower triangles, complex128) of one k-point of the
precision-form workload: cubic cell a = 24 bohr, 128 atoms of 8 types,
R_MT = 2.0, lmax = 10 (L = 121, K = 2 L a = 30976 stacked rows), n_G = 8000,
seeded synthetic inputs (see hybridhsdla_gb300/synth.py, config "c2").

Reported:
  value        effective FP64-equivalent TFLOP/s of the Ozaki-FP8 path with the
               inputs resident in HBM (canonical work 20 G^2 La + 24 L^2 a G per
               k-point, the reference's own flop formulas);
  e2e          the same metric through the C ABI entry point hsdla_create_hs with
               pinned HOST buffers: input upload and the H/S download are inside
               the timed region;
  fp64         the plain FP64 (DMMA) path on the same k-point, and the Ozaki
               path's relative errors against it;
  roofline     the dominant launch (the S/H digit-product contraction) against the
               FP8 tensor peak;
  cpu_baseline the oracle port of the reference CPU path (construct_AB + the
               create_HS2_stripped_v2 BLAS sequence on OpenBLAS), bounded sample.

``--impl reference`` times the reference CPU path (the oracle port: the
reference itself does not build on this image) on a bounded sample of the same
workload, in the same unit.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H+S gen ms/k-point & eff. TFLOP/s: emulated vs native FP64 at ≤1e-13 rel err"
UNIT = "TFLOP/s (FP64-equivalent, 20*G^2*La + 24*L^2*a*G per k-point)"
WORKLOAD = "c2"
WORKLOAD_TEXT = {
    "c0": "c0: cubic a=10 bohr, 4 atoms / 2 types, lmax 6, n_G 500, 1 k-point",
    "c1": "c1: 14x14x20 bohr, 32 atoms / 4 types, lmax 8, n_G 3000, 1 k-point",
    "c2": "c2: cubic a=24 bohr, 128 atoms / 8 types, lmax 10, n_G 8000, 1 k-point",
    "c3": "c3: 17.6x17.6x25.2 bohr, 64 atoms / 4 types, lmax 8, 64 k-points (4x4x4), n_G 6000-6600, CUDA graph",
    "c4": "c4: cubic a=40 bohr, 512 atoms / 16 types, lmax 10, 4 k-points, n_G 19800-20700, CUDA graph",
    "c2t1": "c2t1: c2's cell and n_G 8000 with 16 atoms of one type (one per-type S/H launch of c2's shape)",
    "c2r": "c2r: c2 with per-atom rotations, the atoms of each type in two rotation classes (16 classes)",
}
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "oz_pair_c2.md")


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def _traffic_from_profile():
    """dram bytes per launch of the dominant kernel from the committed ncu summary."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.strip().startswith("traffic_bytes_per_launch_c2:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_kpoints(kpoints, rank: int, world: int):
    """k-points of one replica: rank r takes r, r + N, ... (k-points are independent; the
    reference has no exchange step, so ranks share nothing but the final timing)."""
    return list(kpoints)[rank::world]


def rank_kpoints(kpoints, rank: int, world: int):
    """A batched workload's k-points are split over the replicas; a single-k-point workload runs
    one full copy per replica (weak scaling)."""
    return shard_kpoints(kpoints, rank, world) if len(kpoints) > 1 else list(kpoints)


def bench_config(workload: str, ws: int, kpoints_per_rank: int) -> dict:
    """The workload both arms report (the reference arm prints the same dict)."""
    return {"workload": WORKLOAD_TEXT.get(workload, workload), "kpoints_per_rank": kpoints_per_rank,
            "l2": "inputs larger than L2 (digit planes and per-type products: GBs per k-point; c2 1.6 GB and 16 GB)",
            "parallelism": f"replicas{ws}"}


def cpu_reference_step(sys_, n_g_sample: int, threads: int):
    """The reference CPU path (construct_AB + the create_HS2_stripped_v2 BLAS sequence) on the
    workload's first k-point with its basis truncated to the first n_g_sample G-vectors (all of
    them when n_g_sample >= n_G).  Returns (seconds, flop)."""
    import oracle
    from hybridhsdla_gb300 import synth
    kp = sys_.kpoints[0]
    n = min(n_g_sample, kp.n_g)
    sub = kp if n == kp.n_g else synth.KPoint(k=kp.k, g=kp.g[:n])
    t0 = time.perf_counter()
    oracle.reference_hs(sys_, sub, nthreads=threads)
    return time.perf_counter() - t0, sys_.flop_per_kpoint(n)


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))
    import oracle
    from hybridhsdla_gb300 import synth
    threads = oracle.nthreads_default()
    sys_ = synth.make_system(args.workload)
    ng = args.ref_sample_ng
    for _ in range(args.warmup):
        cpu_reference_step(sys_, ng, threads)
    tot_s, tot_f = 0.0, 0.0
    for _ in range(args.steps):
        s, f = cpu_reference_step(sys_, ng, threads)
        tot_s += s
        tot_f += f
    v = tot_f / tot_s / 1e12
    kp0 = sys_.kpoints[0]
    sample = (f"each step: the workload's first k-point with its basis truncated to the first "
              f"{min(ng, kp0.n_g)} of its {kp0.n_g} G-vectors (full contraction length, {sys_.num_atoms} atoms, "
              f"lmax {sys_.max_lmax}); rate = canonical flops of the sample / its time")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generators, no dataset)",
            "config": bench_config(args.workload, ws, len(rank_kpoints(sys_.kpoints, 0, ws))),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def secondary_workload(ctx, name: str, steps: int, oracle_n: int) -> dict:
    """One more workload on the same GPU: every k-point of it in one plan (k-point groups, one
    launch per stage, captured in a CUDA graph), `steps` timed executions after one warm-up, and
    the first k-point checked on a random subset of its G-vectors against the oracle."""
    import numpy as np
    import torch

    from hybridhsdla_gb300 import synth
    sys_ = synth.make_system(name)
    t0 = time.perf_counter()
    plan = ctx.plan(sys_, precision="ozaki", num_slices=0, use_graph=True)
    outs = plan.alloc_outputs()
    rep = plan.execute(outs)                         # slice autotune, tile tuning, graph capture
    plan.execute(outs)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        rep = plan.execute(outs)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    nk = len(sys_.kpoints)
    flop = sys_.total_flop()
    out = {"workload": WORKLOAD_TEXT.get(name, name), "kpoints": nk, "ms_total": ms, "ms_per_kpoint": ms / nk,
           "value": flop / (ms * 1e-3) / 1e12, "unit": UNIT, "steps": steps, "num_slices": rep["num_slices"],
           "tile_halves": rep["tile_halves"], "merged_units": rep["merged_units"],
           "tile_tuned": rep["tile_tuned"], "kernel_launches": rep["kernel_launches"],
           "setup_s": round(setup_s, 2), "graph": True}
    if oracle_n > 0:
        import oracle
        kp = sys_.kpoints[0]
        idx = np.sort(np.random.default_rng(77).choice(kp.n_g, min(oracle_n, kp.n_g), replace=False))
        Hr, Sr = oracle.reference_hs(sys_, synth.KPoint(k=kp.k, g=kp.g[idx]))
        ti = torch.from_numpy(idx).to(outs[0][0].device)
        errs = {}
        for nm, Xd, R in (("H", outs[0][0], Hr), ("S", outs[0][1], Sr)):
            X = np.tril(Xd.index_select(0, ti).index_select(1, ti).cpu().numpy().T)
            errs[nm + "_fro"], errs[nm + "_max"] = oracle.lower_errors(X, R)
        out["oracle_random_subset"] = {"n": len(idx), "kpoint": 0, **errs}
    plan.close()
    del outs
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch

    from hybridhsdla_gb300 import api, synth

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    ctx = api.Context(dev)
    sys_ = synth.make_system(args.workload)
    batched = len(sys_.kpoints) > 1
    # replicas over k-points: rank r takes k-points r, r + N, ... of a batched workload (weak
    # scaling keeps one full copy of a single-k-point workload per rank)
    kps = rank_kpoints(sys_.kpoints, rank, ws)
    kp = kps[0]
    G = kp.n_g
    flop = sum(sys_.flop_per_kpoint(k.n_g) for k in kps)

    plan = ctx.plan(sys_, kpoints=kps, precision="ozaki", num_slices=args.slices, use_graph=batched)
    outs = plan.alloc_outputs()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        rep = plan.execute(outs)
    torch.cuda.synchronize()
    _barrier(ws)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dom_ms, launches = [], 0
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            rep = plan.execute(outs)
            dom_ms.append(rep["ms_dominant"])
            launches += rep["kernel_launches"]
        ev1.record(stream)
        torch.cuda.synchronize()
    _barrier(ws)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = _max_over_ranks(ws, ms)
    value = ws * flop / (ms * 1e-3) / 1e12
    dominant_flop = rep["dominant_flop"]
    S_oz = outs[0][1].clone()
    H_oz = outs[0][0].clone()
    plan.close()
    del outs

    # ---- end to end through the C ABI with pinned host buffers (first k-point of the rank)
    Hh = torch.empty((G, G), dtype=torch.complex128).pin_memory()
    Sh = torch.empty((G, G), dtype=torch.complex128).pin_memory()
    outs_h = [(Hh.numpy().T, Sh.numpy().T)]          # column-major views of the pinned buffers
    tmats = api.prepare_tmats(sys_)
    ctx.create_hs(sys_, kpoints=[kp], precision="ozaki", num_slices=args.slices, tmats=tmats, out=outs_h)  # warm
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, args.e2e_calls))
    e2e_calls, e2e_dev, e2e_dom, e2e_host = [], [], [], []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tc = time.perf_counter()
        _, rep_e = ctx.create_hs(sys_, kpoints=[kp], precision="ozaki", num_slices=args.slices, tmats=tmats,
                                 out=outs_h)
        e2e_calls.append((time.perf_counter() - tc) * 1e3)
        e2e_dev.append(rep_e["ms_total"])
        e2e_dom.append(rep_e["ms_dominant"])
        e2e_host.append(rep_e["ms_host_setup"])
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = _max_over_ranks(ws, e2e_s)
    e2e_flop = sys_.flop_per_kpoint(G)
    h2d = sum(a.nbytes for a in (kp.g, tmats[0], tmats[1], tmats[2], sys_.u, sys_.u_dr, sys_.dE_u,
                                  sys_.dE_u_dr, sys_.dE_u_norm, sys_.atom_pos, sys_.atom_type, sys_.type_rmt))
    # the end-to-end outputs against the device path's, lower triangles, outside the timed region
    # (its own one-k-point plan: the slice autotuner may choose another digit count, else the same
    # launches give the same bits)
    e2e_vs = {"num_slices": rep_e["num_slices"], "device_path_num_slices": rep["num_slices"]}
    rel, same = 0.0, True
    for Xh, Xd in ((Hh, H_oz), (Sh, S_oz)):
        d = torch.tril(Xh.to(Xd.device).T - Xd.T)      # device buffers are column-major: tensor[col, row]
        rel = max(rel, float(torch.linalg.norm(d) / torch.linalg.norm(torch.tril(Xd.T))))
        same = same and bool(torch.count_nonzero(d) == 0)
        del d
    e2e_vs["rel_fro"] = rel
    e2e_vs["identical"] = same
    if rep_e["outputs_in_place"]:
        # the combine wrote the lower triangles of H and S into the page-locked buffers
        d2h = 2 * 16 * G * (G + 1) // 2
    else:
        # the download copies each 512-column block of H and S from its first row down
        d2h = 2 * 16 * sum((G - c0) * min(512, G - c0) for c0 in range(0, G, 512))

    # ---- plain FP64 path on the first k-point, and the Ozaki error against it
    fp64 = None
    S64 = H64 = None
    if not args.skip_fp64 and rank == 0:
        pl64 = ctx.plan(sys_, kpoints=[kp], precision="fp64")
        o64 = pl64.alloc_outputs()
        r64 = pl64.execute(o64)
        torch.cuda.synchronize()
        H64, S64 = o64[0][0], o64[0][1]

        def errs(X, R):
            Xl = torch.tril(X.transpose(0, 1))
            Rl = torch.tril(R.transpose(0, 1))
            d = Xl - Rl
            return (float(torch.linalg.norm(d) / torch.linalg.norm(Rl)),
                    float(d.abs().max() / Rl.abs().max()))
        eS, eH = errs(S_oz, o64[0][1]), errs(H_oz, o64[0][0])
        fp64 = {"ms_per_kpoint": r64["ms_total"], "tflops": r64["eff_tflops"],
                "dominant_ms": r64["ms_dominant"],
                "ozaki_speedup": r64["ms_total"] / (ms / len(kps)),
                "ozaki_rel_err_vs_fp64": {"S_fro": eS[0], "S_max": eS[1], "H_fro": eH[0], "H_max": eH[1]}}
        pl64.close()
        del o64

    # ---- oracle checks of the first k-point at its full contraction length: an H or S element
    # depends only on the A and B columns of its own two G-vectors, so the oracle run on a subset
    # of the G-vectors gives exactly the sub-matrix H[sub, sub], S[sub, sub] (sub in ascending
    # order keeps the lower triangle lower).  Two subsets: the leading block and a seeded random one.
    block = None
    if args.oracle_block > 0 and rank == 0:
        import oracle
        nb = min(args.oracle_block, G)
        rng = np.random.default_rng(1234)
        subsets = {"leading": np.arange(nb), "random": np.sort(rng.choice(G, nb, replace=False))}
        block = {"n": nb, "note": "relative Frobenius / max-norm error of the lower triangle of H[sub, sub] and "
                                  "S[sub, sub] against the oracle run on those G-vectors (full contraction length)"}
        for sname, idx in subsets.items():
            sub = synth.KPoint(k=kp.k, g=kp.g[idx])
            t_or = time.perf_counter()
            Hr, Sr = oracle.reference_hs(sys_, sub)
            t_or = time.perf_counter() - t_or
            ti = torch.from_numpy(idx).to(H_oz.device)
            for prec, Hd, Sd in (("ozaki", H_oz, S_oz), ("fp64", H64, S64)):
                if Hd is None:
                    continue
                ent = block.setdefault(prec, {}).setdefault(sname, {})
                for nm, Xd, R in (("H", Hd, Hr), ("S", Sd, Sr)):
                    X = np.tril(Xd.index_select(0, ti).index_select(1, ti).cpu().numpy().T)
                    fro, mx = oracle.lower_errors(X, R)
                    ent[nm + "_fro"], ent[nm + "_max"] = fro, mx
            block.setdefault("oracle_s", {})[sname] = round(t_or, 2)
        worst = max(v for p in ("ozaki", "fp64") for e in block.get(p, {}).values() for v in e.values())
        block["max_err"] = worst
        block["within_1e-13"] = worst <= 1e-13

    peaks, src = _peaks()
    fp8_peak = 2.0 * peaks["bf16_tflops"]
    dom = float(np.median(dom_ms))
    achieved = dominant_flop / (dom * 1e-3) / 1e12
    traffic = _traffic_from_profile() if args.workload == "c2" else None
    roof = {"bound": "tensor", "achieved": achieved, "peak": fp8_peak, "unit": "TFLOP/s",
            "frac": achieved / fp8_peak, "traffic": traffic,
            "kernel": "oz_pair_kernel (one type's S and H lower-triangle digit products per launch, "
                      "CTA-pair 256x256 tiles; achieved and traffic per launch)",
            "peak_source": f"2 x {src} bf16 burst (FP8 e4m3 dense rate = 2x bf16 on tcgen05)"}

    cpu = None
    if not args.skip_cpu and rank == 0:
        import oracle
        os.environ.setdefault("OPENBLAS_NUM_THREADS", str(os.cpu_count() or 1))
        threads = oracle.nthreads_default()
        cpu_reference_step(sys_, args.ref_sample_ng, threads)       # warm
        s_, f_ = cpu_reference_step(sys_, args.ref_sample_ng, threads)
        samp = {"value": f_ / s_ / 1e12, "seconds": round(s_, 2),
                "sample": f"first k-point with its basis truncated to the first {min(args.ref_sample_ng, G)} "
                          f"G-vectors (the reference arm's step)"}
        if args.cpu_full:
            sf_, ff_ = cpu_reference_step(sys_, G, threads)
            cpu = {"value": ff_ / sf_ / 1e12, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"one full k-point of the workload (n_G {G}, all {sys_.num_atoms} atoms, lmax "
                             f"{sys_.max_lmax}): {sf_:.1f} s", "ms_per_kpoint": sf_ * 1e3,
                   "truncated_sample": samp}
        else:
            cpu = {"value": samp["value"], "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": samp["sample"] + f", {s_:.1f} s"}

    # ---- the batching and large combined workloads on the same GPU (evidence beside the headline)
    extra = {}
    if rank == 0 and ws == 1:
        for name in [w for w in args.also.split(",") if w]:
            try:
                extra[name] = secondary_workload(ctx, name, args.also_steps, args.also_oracle)
            except Exception as exc:      # reported, not fatal: the headline line still prints
                extra[name] = {"error": f"{type(exc).__name__}: {exc}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators, no dataset)",
                "config": bench_config(args.workload, ws, len(kps)),
                "precision": f"ozaki-fp8 e4m3, {rep['num_slices']} digit slices",
                "ms_per_kpoint": ms / len(kps),
                "e2e": {"value": ws * e2e_flop / e2e_s / 1e12, "unit": UNIT, "ms_per_kpoint": e2e_s * 1e3,
                        "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                        "calls_ms": [round(x, 2) for x in e2e_calls],
                        "calls_device_ms": [round(x, 2) for x in e2e_dev],
                        # per call, the device time of the S/H product launches alone (no host
                        # traffic): a slow call whose products kept their time was slowed on the
                        # host side or its link
                        "calls_dominant_ms": [round(x, 2) for x in e2e_dom],
                        # per call, the host's plan creation and set-up before the first launch
                        "calls_host_setup_ms": [round(x, 2) for x in e2e_host],
                        "median_ms": float(np.median(e2e_calls)),
                        "outputs": ("written in place by the combine in %d column blocks while the products "
                                    "of the next block ran" % rep_e["output_blocks"]) if rep_e["output_blocks"]
                        else "written in place by the last combine" if rep_e["outputs_in_place"]
                        else "downloaded by the copy engine",
                        "vs_device_path": e2e_vs,
                        "note": "hsdla_create_hs on the rank's first k-point, pinned host buffers; "
                                "value = mean over calls_ms"},
                "gpu_launches": launches,
                "tiles": {"halves": rep["tile_halves"], "merged_units": rep["merged_units"],
                          "tuned": rep["tile_tuned"], "row_sets": rep["num_row_sets"],
                          "rotation_classes": rep["rotation_classes"]},
                "stage_ms": {"construct_ab": rep["ms_construct_ab"], "tapply": rep["ms_tapply"],
                             "contract": rep["ms_contract"], "dominant": dom},
                "fp64": fp64, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary()}
        if block is not None:
            line["oracle_block"] = block
        if extra:
            line["workloads"] = extra
        if rep.get("num_panels", 1) > 1:
            line["config"]["atom_panels"] = rep["num_panels"]
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--slices", type=int, default=0, help="Ozaki digit slices (0 = default)")
    ap.add_argument("--ref-sample-ng", type=int, default=3200)   # ~11 s of CPU work per step
    ap.add_argument("--oracle-block", type=int, default=1024,
                    help="compare N x N sub-matrices of the first k-point's H and S (the leading block and a "
                         "seeded random subset of G-vectors) with the oracle; 0 = off")
    ap.add_argument("--cpu-full", type=int, default=1,
                    help="1: time the reference CPU path on one full k-point of the workload once")
    ap.add_argument("--e2e-calls", type=int, default=8, help="end-to-end calls through hsdla_create_hs")
    ap.add_argument("--also", default="c3,c4",
                    help="further workloads timed after the headline (comma list; empty = none)")
    ap.add_argument("--also-steps", type=int, default=2)
    ap.add_argument("--also-oracle", type=int, default=256,
                    help="random-subset size of the oracle check of each further workload's first k-point")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOAD_TEXT),
                    help="workload (default: the c2 precision-form case the metric is quoted on)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
