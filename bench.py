#!/usr/bin/env python
"""Omega evaluations per second of the GB300 cluster-ED path.

Workload: the 4x3 square Hubbard cluster (Ns=12, Nspin=2, U=8, xmu=4) with a
variational antiferromagnetic Weiss field M swept over 16 points in [0, 0.3],
a 32x32 k-grid in the reduced zone, 200-step Green's function chains for every
site and spin, and the Potthoff Omega integrated on the imaginary axis with an
8192-node rule.  One step = one full vca_solve (all 169 sectors diagonalised,
all chains, Omega) at the next M of the sweep.  Synthetic inputs restated from
the reference's square-lattice driver recipe (no dataset exists).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` = Omega evals/s with Hk resident in HBM (CUDA events on the library
stream); `e2e` = the same through vca_gpu_solve with host buffers (Hk and Hloc
copied in, Omega copied out every step).  N > 1 (torchrun) runs independent
replicas over different M (weak scaling, no data-path collective).
`--impl reference` times the CPU restatement of the reference path on the
host cores (the Fortran reference does not build on this image).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Omega evals/sec (plain GPU path, |dOmega|<=1e-10 vs FP64 oracle)"
# the arithmetic the timed path runs: the 4x3 Hubbard Hamiltonian is real with
# one hopping magnitude, so the Lanczos vectors are int64 fixed point (2^-59)
# with exact int128 dot products, the scalars and Omega FP64
DTYPE = "fx64 vectors (Q59, int128 dots) / f64 scalars and Omega"
DTYPE_REF = "f64"
UNIT = "Omega evals/s"
WORKLOAD = ("square4x3 Hubbard U=8 Nspin=2, M_AF sweep 16 pts [0,0.3], 32x32 k-grid, "
            "200-step GF chains (chan4), 8192-node Omega rule")


def dist_env():
    from vca_gb300.replicas import dist_env as _d
    return _d()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_traffic(name: str):
    """dram bytes per launch recorded in a committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def build_points():
    import numpy as np
    from vca_gb300 import clusters
    ms = np.linspace(0.0, 0.3, 16)
    return [clusters.square(nx=4, ny=3, U=8.0, xmu=4.0, maf=float(m), nspin=2, nkx=32, nky=32,
                            ngfiter=200, omega_nodes=8192) for m in ms]


# ---------------------------------------------------------------------------
# CPU timing of the oracle on a bounded sample of one Omega evaluation
# ---------------------------------------------------------------------------
def cpu_sample(pt, threads: int):
    """(estimated Omega evals/s, description, estimated seconds per eval,
    measured seconds of the sample).  Each stage is sampled in the parallel
    form the oracle's full evaluation runs it in: sectors diagonalised one per
    thread (the `threads` largest, scaled by total/sampled dimension), chains
    one per thread (`threads` 200-step chains on the GF target sector, scaled
    by chains/threads), and the frequency rule's k-sums parallel over k (8 of
    the nodes, scaled by the node count)."""
    import numpy as np
    from oracle import oracle as orc
    from oracle.oracle import Oracle
    orc.set_threads(threads)
    o = Oracle.from_point(pt)
    Ns = o.Ns
    tgt = 1 + 6 + 7 * (Ns + 1)         # GF target sector (7,6), dim 731,808
    t_all = time.perf_counter()
    dims = np.array([o.dim(s) for s in range(1, o.Nsectors + 1)], dtype=np.float64)
    big = np.argsort(-dims, kind="stable")[:threads]
    mask = np.zeros(o.Nsectors, dtype=np.int32)
    mask[big] = 1
    t0 = time.perf_counter()
    o.diagonalize(mask)
    t_gs = time.perf_counter() - t0
    gs_total = t_gs * dims.sum() / dims[big].sum()
    t_chain = o.chain_sample(tgt, threads, 200)
    L = pt.cfg.Nlat * pt.cfg.Norb
    chains = pt.cfg.Nspin * (2 * L + 4 * L * (L - 1))
    nn = 8
    t0 = time.perf_counter()
    for w in np.linspace(0.1, 5.0, nn):
        o.sum_kmesh(float(w))
    t_node = (time.perf_counter() - t0) / nn
    total = gs_total + chains / threads * t_chain + pt.cfg.omega_nodes * t_node
    sample = (f"oracle (C++/OpenMP restatement) on {threads} threads, each stage in the evaluation's own "
              f"parallel form: the {len(big)} largest of {o.Nsectors} sectors diagonalised one per thread "
              f"[{t_gs:.2f}s] scaled by total/sampled dimension; {threads} of {chains} 200-step chains on "
              f"sector (7,6), one per thread [{t_chain:.2f}s]; {nn} of {pt.cfg.omega_nodes} Omega nodes "
              f"[{t_node * 1e3:.1f}ms each]; one eval estimated at {total:.0f}s")
    return 1.0 / total, sample, total, time.perf_counter() - t_all


def run_reference(args):
    """The reference arm: the oracle port (the Fortran reference does not
    build here) on all host threads.  One step is one bounded sample of an
    Omega evaluation at the benchmark configuration, each stage in the
    evaluation's own parallel form (the largest sectors' ground states one per
    thread, one chain per thread, 8 of the 8192 Omega nodes; cpu_sample);
    ms_per_step is that sample's measured wall time, and value the Omega
    evals/s the sample implies (its parts scaled to a whole evaluation)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    pts = build_points()
    vals, walls = [], []
    sample = ""
    est = 0.0
    for s in range(args.warmup + args.steps):
        v, sample, est, wall = cpu_sample(pts[s % len(pts)], threads)
        if s >= args.warmup:
            vals.append(v)
            walls.append(wall)
    value = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(walls) / len(walls),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE_REF,
        "data": "synthetic", "config": {"workload": WORKLOAD, "parallelism": "host threads",
                                        "step": "one bounded sample of an Omega evaluation"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "estimated_seconds_per_eval": round(est, 1)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def hxv_operand(s, D, m, dimup):
    """Unit-norm random columns in the library's arithmetic (FP64, or int64
    fixed point with scale 2^-F when the fixed-point path is active), and the
    name of the kernel the library runs on them."""
    import torch
    fx, F, _ = s.arith_info()
    x = torch.randn(D, m, dtype=torch.float64, device="cuda")
    x /= torch.linalg.vector_norm(x, dim=0, keepdim=True)
    if fx:
        # hxv_variant 2: the chains' layout (rows in hop-count order) and
        # kernel; 0: staged form while the up block fits; 1: warp form
        fits = m >= 16 and dimup * 8 * 8 <= 100 * 1024
        v = s.cfg.hxv_variant
        if m < 16:
            name = "k_hxv_fx"
        elif v == 2:
            name = "k_hxv_fx_r"
        elif v == 0 and fits:
            name = "k_hxv_fx_s"
        else:
            name = "k_hxv_fx_w"
        return torch.round(x * 2.0 ** F).to(torch.int64).reshape(-1), name
    return x.reshape(-1), "k_hxv_real"


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    rank, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    import numpy as np
    from vca_gb300 import build as vbuild
    vbuild.build()
    from vca_gb300.solver import VcaSolver

    from vca_gb300.replicas import Group, partition
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    grp = Group(dist)
    barrier, allmax = grp.barrier, grp.max

    pts = build_points()
    mine = [pts[i] for i in partition(len(pts), rank, world)]
    cfg0 = mine[0].cfg.copy()
    cfg0.hxv_variant = 2  # the roofline H x v runs in the chains' layout and kernel
    s = VcaSolver(cfg0)
    s.upload_hk(mine[0].Hk)
    for i in range(args.warmup):
        s.solve_resident(mine[i % len(mine)].Hloc)
    stage_ms = s.timings().tolist()
    # ---- value: Hk resident, device time on the library stream ----------
    clocks = ClockSampler(0 if world > 1 else local)
    barrier()
    s.synchronize()
    l0 = s.kernel_launches()
    s.timer_start()
    omegas = []
    for i in range(args.steps):
        omegas.append(s.solve_resident(mine[(args.warmup + i) % len(mine)].Hloc))
    ms = s.timer_stop()
    launches = s.kernel_launches() - l0
    barrier()
    ck = clocks.stop()
    ms = allmax(ms)
    value = args.steps * world / (ms / 1e3)
    # ---- e2e: host buffers through vca_gpu_solve ------------------------
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        p = mine[(args.warmup + i) % len(mine)]
        s.solve(p.Hloc, p.Hk)
    e2e_s = allmax(time.perf_counter() - t0)
    e2e = args.steps * world / e2e_s
    p0 = mine[0]
    h2d = int(p0.Hloc.nbytes + p0.Hk.nbytes)
    # ---- roofline of the dominant kernel: batched real H x v on the chain
    # target sector (7,6) with the particle batch of one spin (408 columns)
    roof = None
    if rank == 0:
        import torch
        isec = 1 + 6 + 7 * 13
        _, _, du, dd = s.sector_info(isec)
        D = du * dd
        L = 12
        m = L + L * (L - 1) + 2 * L * (L - 1)
        x, kname = hxv_operand(s, D, m, du)
        y = torch.empty_like(x)
        torch.cuda.synchronize()
        reps = 5
        t_ms = s.hxv_timed(isec, x.data_ptr(), y.data_ptr(), 0, m, reps)
        bytes_alg = 16.0 * D * m
        peak, kind = measured_peaks()
        ach = bytes_alg / (t_ms / 1e3) / 1e9
        traffic = profile_traffic(kname.split("+")[0].replace("k_", "") + "_square4x3.md")
        roof = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "traffic": traffic,
                "kernel": kname, "launch_ms": round(t_ms, 4),
                "algorithmic_bytes_per_launch": bytes_alg,
                "peak_kind": kind,
                "shape": f"sector (7,6) D={D}, {m} real columns"}
        del x, y
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": DTYPE, "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (chain column batches 2.3 GB per buffer)",
                   "stage_ms_last_warmup": [round(x, 1) for x in stage_ms]},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8},
        "gpu_launches": int(launches),
        "clocks": ck,
        "omega_samples": [round(x, 12) for x in omegas[:3]],
    }
    if roof is not None:
        out["roofline"] = roof
    if rank == 0:
        out["accuracy"] = accuracy_check(pts, cfg0)
    if rank == 0:
        # single-vector H x v on the half-filled 4x4 sector (the largest
        # sector of the 4x4 cluster), the vector size the roofline target
        # of this path is stated for; measured after the solves (it replaces
        # the library context)
        s.close()
        out["hxv_single_4x4"] = hxv_single_4x4()
        out["finite_t"] = finite_t_sample(cpu=(world == 1 and not args.no_cpu))
        out["batched_c3"] = batched_block("c3", args.batch_c3, 8, 3)
        out["batched_c4"] = batched_block("c4", args.batch_c4, 8, 3)
        out["surrogate_search"] = search_block()
    if rank == 0 and world == 1 and not args.no_cpu:
        v, sample, _, _ = cpu_sample(pts[0], os.cpu_count() or 1)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": sample}
    if rank == 0:
        print(json.dumps(out))
    else:
        s.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def accuracy_check(pts, cfg0, idx: int = 5) -> dict:
    """Omega of sweep point idx (M = 0.1) in the timed arithmetic and in FP64,
    and against the oracle's value at exactly this configuration
    (tests/golden/config_c2_m05.npz, written by tests/golden/make_golden.py)."""
    import numpy as np
    from vca_gb300.solver import VcaSolver
    p = pts[idx]
    vals = {}
    for name, arith in (("timed", cfg0.arith), ("fp64", 1)):
        cfg = cfg0.copy()
        cfg.arith = arith
        s = VcaSolver(cfg)
        vals[name] = s.solve(p.Hloc, p.Hk)
        s.close()
    rel = lambda a, b: abs(a - b) / max(1.0, abs(b))  # noqa: E731
    out = {"point": f"M = {p.params['maf']:.4f}", "omega": vals["timed"],
           "omega_fx_vs_fp64": rel(vals["timed"], vals["fp64"])}
    gold = os.path.join(ROOT, "tests", "golden", f"config_c2_m{idx:02d}.npz")
    if os.path.exists(gold):
        out["omega_vs_oracle_fixture"] = rel(vals["timed"], float(np.load(gold)["sft"]))
    return out


def finite_t_point():
    from vca_gb300 import clusters
    return clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=100,
                           omega_nodes=256, lanc_nstates_total=2, beta=20.0, bandwidth=8.0)


def finite_t_sample(reps: int = 3, cpu: bool = True) -> dict:
    """Finite-temperature solves (LANC_NSTATES_TOTAL = 2, beta = 20) of the
    3x3 Hubbard cluster with a Weiss field, 8x8 k-grid: GPU wall time per
    vca_gpu_solve (host buffers) after one warm-up, and, on one process, the
    oracle's time for the same solve on all host cores."""
    from vca_gb300.solver import VcaSolver
    pt = finite_t_point()
    s = VcaSolver(pt.cfg)
    om = s.solve(pt.Hloc, pt.Hk)
    t0 = time.perf_counter()
    for _ in range(reps):
        om = s.solve(pt.Hloc, pt.Hk)
    gpu_ms = (time.perf_counter() - t0) * 1e3 / reps
    th = s.thermal()
    nst = len(s.states())
    s.close()
    out = {"workload": "3x3 Hubbard U=8 xmu=4 M=0.1, Nspin=2, 8x8 k, 100-step chains, beta=20",
           "gpu_ms_per_solve": round(gpu_ms, 2), "omega": om, "states": nst,
           "nmax": th["nmax"], "contour_points": th["contour_points"]}
    if cpu:
        from oracle import oracle as orc
        from oracle.oracle import Oracle
        threads = orc.set_threads(os.cpu_count() or 1)
        o = Oracle.from_point(pt)
        t0 = time.perf_counter()
        ref = o.solve()[0]
        out["cpu_oracle_ms_per_solve"] = round((time.perf_counter() - t0) * 1e3, 1)
        out["cpu_cores"] = threads
        out["omega_rel_diff"] = abs(om - ref) / abs(ref)
    return out


def batch_points(which: str, B: int):
    """The first B points of the C3 batch (2x2 cluster + 8 bath levels, U=4,
    24x24 k, 200-step chains, 4096-node rule) or of the C4 batch (BHZ 2x2,
    Norb=2, Nspin=2, 48x48 k, 200-step chains, 4096-node rule), Hk shared."""
    import numpy as np
    from vca_gb300 import clusters
    if which == "c3":
        pts = clusters.batch_square_bath(B=B)
        desc = "C3: 2x2 Hubbard + 8 bath levels, U=4, 24x24 k, 200-step chains, 4096 nodes"
    else:
        rng = np.random.Generator(np.random.PCG64(20261203 + 4))
        prm = rng.uniform([1.5, -0.2], [2.5, 0.2], size=(B, 2))
        base = clusters.bhz(mass=2.0, delta=0.0)  # H_k (48x48) is the same for every point
        pts = [clusters.bhz(mass=p[0], delta=p[1], nk1=1) for p in prm]
        for p in pts:
            p.Hk = base.Hk
        desc = "C4: BHZ 2x2, Norb=2, Nspin=2, 48x48 k, 200-step chains, 4096 nodes"
    return pts, desc


def _nsectors(cfg) -> int:
    ns = cfg.Nlat * cfg.Norb + cfg.Nlat_bath * cfg.Norb_bath
    return (ns + 1) ** 2


def _solve_points(pts, batch_loop: int, sector_at_a_time: int = 0):
    import numpy as np
    from vca_gb300.solver import VcaSolver
    cfg = pts[0].cfg.copy()
    cfg.batch_loop, cfg.sector_at_a_time = batch_loop, sector_at_a_time
    s = VcaSolver(cfg, pts[0].bath_h, pts[0].bath_v)
    s.solve(pts[0].Hloc, pts[0].Hk, pts[0].bath_h, pts[0].bath_v)  # warm-up (Hk upload, node rule)
    Hl = np.stack([p.Hloc for p in pts], axis=-1)
    bh = np.stack([p.bath_h for p in pts], axis=-1) if pts[0].bath_h is not None else None
    bv = np.stack([p.bath_v for p in pts], axis=-1) if pts[0].bath_v is not None else None
    s.synchronize()
    t0 = time.perf_counter()
    om = s.solve_batch(Hl, pts[0].Hk, bh, bv)
    dt = time.perf_counter() - t0
    stages = s.timings(batched=not batch_loop)
    s.close()
    return om, dt, stages


def batched_block(which: str, B: int, n_loop: int, n_sat: int) -> dict:
    """Omega evals/s of the batched form (vca_gpu_solve_batch, B points in
    one call) against the plain path on the same points: one point after
    another through the per-point path (every sector of a point in one
    batched search), and the reference's loop structure (one sector per
    Lanczos run).  Host arrays in, Omega out; wall time of the call."""
    pts, desc = batch_points(which, B)
    # the plain paths run on points spread evenly over the batch (the points'
    # ground states, and so their chains, differ from point to point)
    il = [round(i * (B - 1) / max(1, n_loop - 1)) for i in range(n_loop)]
    isat = [round(i * (B - 1) / max(1, n_sat - 1)) for i in range(n_sat)]
    om_b, t_b, st_b = _solve_points(pts, 0)
    om_l, t_l, _ = _solve_points([pts[i] for i in il], 1)
    om_s, t_s, _ = _solve_points([pts[i] for i in isat], 1, 1)
    d_loop = max(abs(om_b[i] - b) / max(1.0, abs(b)) for i, b in zip(il, om_l))
    d_sat = max(abs(om_b[i] - b) / max(1.0, abs(b)) for i, b in zip(isat, om_s))
    v_b, v_l, v_s = B / t_b, n_loop / t_l, n_sat / t_s
    return {"workload": desc, "unit": "Omega evals/s",
            "batched": {"points": B, "value": round(v_b, 4), "ms_per_eval": round(1e3 * t_b / B, 2),
                        "stage_ms": dict(zip(["tables", "search", "eigenvectors", "chains", "omega",
                                              "closing_plain_solve"], [round(x, 1) for x in st_b[:6]])),
                        "sector_searches_skipped_by_bound": int(st_b[6]),
                        "chain_tile_shape": {"rows_per_tile": int(st_b[7]), "row_lanes_per_block": int(st_b[8]),
                                             "chosen_by": "autotuner"},
                        "sector_searches_total": B * _nsectors(pts[0].cfg)},
            "plain_per_point": {"points": il, "value": round(v_l, 4), "ms_per_eval": round(1e3 * t_l / n_loop, 2),
                                "what": "one point after another, every sector of a point in one batched search"},
            "plain_sector_at_a_time": {"points": isat, "value": round(v_s, 4),
                                       "ms_per_eval": round(1e3 * t_s / n_sat, 2),
                                       "what": "one point and one sector at a time (the reference's loops)"},
            "ratio_vs_sector_at_a_time": round(v_b / v_s, 2), "ratio_vs_per_point": round(v_b / v_l, 2),
            "max_rel_dOmega_vs_plain": max(d_loop, d_sat)}


def search_block() -> dict:
    """Stationary-point searches of Omega over (t', M_AF, staggered charge
    field) of the 2x2 Hubbard cluster (U=8, half filling, 8x8 k, 100-step
    chains, 512 nodes): the plain Newton search (central differences of
    plain solves), the drivers' one-parameter Brent cycled over the
    parameters, and the surrogate-guided search (the network trained on the
    GPU on solver values and forward-difference gradients); every Omega is a
    plain FP64 solve, counted."""
    import numpy as np
    from vca_gb300 import clusters
    from vca_gb300.solver import VcaSolver
    from vca_gb300.surrogate import CountingSolver, coordinate_brent_search, newton_fd_search, surrogate_search
    lo, hi = clusters.SEARCH_LO, clusters.SEARCH_HI
    p0 = 0.5 * (lo + hi)
    pt = clusters.search_point(p0)
    s = VcaSolver(pt.cfg)
    s.upload_hk(pt.Hk)

    def solve(p):
        return s.solve_resident(clusters.search_point(p).Hloc)
    out = {"workload": "2x2 Hubbard U=8 half filling, Nspin=2, 8x8 k, 100-step chains, 512 nodes; "
                       "box t' in [1.1,1.7], M_AF in [0.2,0.55], charge field in [-0.2,0.2]"}
    f = CountingSolver(solve)
    t0 = time.perf_counter()
    p_n, om_n, it = newton_fd_search(f, p0, lo, hi)
    out["plain_newton"] = {"calls": f.calls, "iterations": it, "omega": om_n, "point": p_n.tolist(),
                           "s": round(time.perf_counter() - t0, 2)}
    f = CountingSolver(solve)
    t0 = time.perf_counter()
    p_b, om_b, cyc = coordinate_brent_search(f, p0, lo, hi, ["min", "min", "max"])
    out["plain_coordinate_brent"] = {"calls": f.calls, "cycles": cyc, "dOmega": om_b - om_n,
                                     "s": round(time.perf_counter() - t0, 2)}
    f = CountingSolver(solve)
    t0 = time.perf_counter()
    p_s, om_s, hist = surrogate_search(f, lo, hi, p0, n_design=10, steps=4000)
    out["surrogate"] = {"calls": f.calls, "omega": om_s, "dOmega_vs_newton": om_s - om_n, "point": p_s.tolist(),
                        "s": round(time.perf_counter() - t0, 2),
                        "rounds": [{"dOmega": h["omega"] - om_n, "surrogate_error": h["surrogate_error"],
                                    "omega_gap_estimate": h["omega_gap_estimate"]} for h in hist]}
    out["calls_ratio_vs_newton"] = round(out["plain_newton"]["calls"] / f.calls, 2)
    out["calls_ratio_vs_coordinate_brent"] = round(out["plain_coordinate_brent"]["calls"] / f.calls, 2)
    s.close()
    return out


def hxv_single_4x4(reps: int = 10) -> dict:
    """One H x v of a unit vector on sector (8,8) of the 4x4 Hubbard cluster
    (D = 12870^2 = 165,636,900), CUDA events on the library stream;
    algorithmic bytes 16*D (read v, write Hv).  The paired-column form (the
    library's) and the one-column form (hxv_variant 1) on the same vector;
    their outputs must agree bit for bit."""
    import torch
    from vca_gb300 import clusters
    from vca_gb300.solver import VcaSolver
    pt = clusters.square(nx=4, ny=4, U=8.0, xmu=4.0, maf=0.0, nspin=1, nkx=4, nky=4, ngfiter=10,
                         omega_nodes=64)
    isec = 1 + 8 + 8 * 17
    peak, kind = measured_peaks()
    out = {"sector": [8, 8], "peak": peak, "peak_kind": kind}
    x = y = y0 = None
    for variant, name, kernels in ((0, "paired", "k_hxv1_up2 + k_hxv1_dw2"), (1, "one_column", "k_hxv1_up + k_hxv1_dw")):
        cfg = pt.cfg.copy()
        cfg.hxv_variant = variant
        s4 = VcaSolver(cfg)
        s4.set_hamiltonian(pt.Hloc)
        _, _, du, dd = s4.sector_info(isec)
        D = du * dd
        fx, F, _ = s4.arith_info()
        if x is None:
            g = torch.Generator(device="cuda").manual_seed(4)
            x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
            x /= torch.linalg.vector_norm(x)
            if fx:
                x = torch.round(x * 2.0 ** F).to(torch.int64)
            y = torch.empty_like(x)
        ms = s4.hxv_timed(isec, x.data_ptr(), y.data_ptr(), 0, 1, reps)
        s4.close()
        gbs = 16.0 * D / (ms / 1e3) / 1e9
        out["D"] = D
        out["arith"] = "fx" if fx else "f64"
        out[name] = {"kernels": kernels, "launch_ms": round(ms, 4), "achieved_GBps": round(gbs, 1),
                     "frac": round(gbs / peak, 4)}
        if y0 is None:
            y0 = y.clone()
        else:
            out["bit_identical"] = bool(torch.equal(y0, y))
    # headline fields: the library's form
    out.update({"launch_ms": out["paired"]["launch_ms"], "kernels": out["paired"]["kernels"],
                "achieved_GBps": out["paired"]["achieved_GBps"], "frac": out["paired"]["frac"]})
    del x, y, y0
    return out


def hxv_cols_4x4(ncols: int, reps: int) -> dict:
    """Column-batch H x v on a Green's-function target sector of the 4x4
    cluster (sector (9,8): 11440 x 12870 = 147,232,800), `ncols` slab-major
    int64 columns, CUDA events on the library stream: the slab-pair form
    (the library's) against the warp form (hxv_variant 1), same input;
    algorithmic bytes 16 per element and column."""
    import torch
    from vca_gb300 import clusters
    from vca_gb300.solver import VcaSolver
    pt = clusters.square(nx=4, ny=4, U=8.0, xmu=4.0, maf=0.15, nspin=2, nkx=2, nky=2, ngfiter=10,
                         omega_nodes=64)
    isec = 1 + 9 + 8 * 17
    peak, kind = measured_peaks()
    out = {"sector": [9, 8], "ncols": ncols, "peak": peak, "peak_kind": kind}
    x = y = y0 = None
    for variant, name in ((0, "slab_pair"), (1, "warp")):
        cfg = pt.cfg.copy()
        cfg.hxv_variant = variant
        s = VcaSolver(cfg)
        s.set_hamiltonian(pt.Hloc)
        _, _, du, dd = s.sector_info(isec)
        D = du * dd
        if x is None:
            fx, F, _ = s.arith_info()
            g = torch.Generator(device="cuda").manual_seed(5)
            x = torch.randn(D * ncols, dtype=torch.float64, device="cuda", generator=g)
            x = x.mul_(2.0 ** F / (D ** 0.5 * 4.0)).round_().to(torch.int64)
            y = torch.empty_like(x)
        ms = s.hxv_timed(isec, x.data_ptr(), y.data_ptr(), 0, ncols, reps)
        s.close()
        gbs = 16.0 * D * ncols / (ms / 1e3) / 1e9
        out["D"] = D
        out[name] = {"launch_ms": round(ms, 3), "ms_per_column": round(ms / ncols, 4),
                     "achieved_GBps": round(gbs, 1), "frac": round(gbs / peak, 4)}
        if y0 is None:
            y0 = y.clone()
        else:
            out["bit_identical"] = bool(torch.equal(y0, y))
    del x, y, y0
    return out


def c5_solve(steps: int) -> dict:
    """One plain vca_solve of the 4x4 Hubbard cluster (Ns = 16, 289 sectors,
    largest 12870^2): U = 8, half filling, t' = 1, M_AF = 0.15, Nspin = 2,
    16x16 k-grid, `steps`-step chains (the reference's channel set: 1984
    chains), 8192-node Omega rule; wall time and the library's stage times."""
    import numpy as np
    from vca_gb300 import clusters
    from vca_gb300.solver import VcaSolver
    pt = clusters.square(nx=4, ny=4, U=8.0, xmu=4.0, t=1.0, tprime=1.0, maf=0.15, nspin=2, nkx=16, nky=16,
                         ngfiter=steps, omega_nodes=8192)
    s = VcaSolver(pt.cfg)
    t0 = time.perf_counter()
    om = s.solve(pt.Hloc, pt.Hk)
    dt = time.perf_counter() - t0
    st = s.timings()
    out = {"workload": "C5: 4x4 Hubbard U=8, half filling, t'=1, M_AF=0.15, Nspin=2, 16x16 k, "
                       f"{steps}-step chains (chan4), 8192-node Omega rule",
           "omega": om, "seconds": round(dt, 2),
           "stage_s": {"hamiltonian": round(st[0] / 1e3, 3), "diagonalize": round(st[1] / 1e3, 3),
                       "chains": round(st[2] / 1e3, 3), "omega": round(st[3] / 1e3, 3)},
           "arith": "fx" if s.arith_info()[0] else "f64"}
    cs, cl, nb = s.chain_timings()
    out["chain_stage"] = {"start_vectors_s": round(cs / 1e3, 3), "lanczos_steps_s": round(cl / 1e3, 3),
                          "column_batches": nb}
    out["egs"] = s.energies()[0]
    out["states"] = [list(x) for x in s.states()]
    s.close()
    return out


def profile_hxv(ncols: int, reps: int, variant: int = 0, pairing: bool = True) -> int:
    """Batched H x v only (for ncu captures of the H x v kernel)."""
    import torch
    from vca_gb300 import build as vbuild
    vbuild.build()
    from vca_gb300.solver import VcaSolver
    pt = build_points()[5]
    cfg = pt.cfg.copy()
    cfg.hxv_variant = variant
    s = VcaSolver(cfg)
    s.set_hop_pairing(pairing)
    s.set_hamiltonian(pt.Hloc)
    isec = 1 + 6 + 7 * 13
    _, _, du, dd = s.sector_info(isec)
    D = du * dd
    x, kname = hxv_operand(s, D, ncols, du)
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    ms = s.hxv_timed(isec, x.data_ptr(), y.data_ptr(), 0, ncols, reps)
    print(json.dumps({"kernel": kname, "sector": [7, 6], "D": D, "ncols": ncols, "reps": reps, "hop_pairing": pairing,
                      "ms_per_launch": ms, "alg_GBps": 16.0 * D * ncols / (ms / 1e3) / 1e9}))
    s.close()
    return 0


def profile_batch(which: str, points: int, autotune: bool) -> int:
    """Batched form on the first points of the C3 or C4 batch (FP64), then one
    plain solve of the first point (for ncu captures of the batched kernels)."""
    import numpy as np
    from vca_gb300 import build as vbuild
    vbuild.build()
    from vca_gb300.solver import VcaSolver
    pts, _ = batch_points(which, points)
    Hl = np.stack([p.Hloc for p in pts], axis=-1)
    bh = np.stack([p.bath_h for p in pts], axis=-1) if pts[0].bath_h is not None else None
    bv = np.stack([p.bath_v for p in pts], axis=-1) if pts[0].bath_v is not None else None
    cfg = pts[0].cfg.copy()
    cfg.arith = 1
    s = VcaSolver(cfg, pts[0].bath_h, pts[0].bath_v)
    s.set_autotune(autotune)
    t0 = time.perf_counter()
    om = s.solve_batch(Hl, pts[0].Hk, bh, bv)
    tb = time.perf_counter() - t0
    stages = s.timings(batched=True).tolist()
    t0 = time.perf_counter()
    o1 = s.solve(pts[0].Hloc, pts[0].Hk, pts[0].bath_h, pts[0].bath_v)
    print(json.dumps({"batched_s": tb, "batched_stage_ms": stages, "plain_s": time.perf_counter() - t0,
                      "plain_stage_ms": s.timings().tolist(), "omega0": [float(om[0]), o1]}))
    s.close()
    return 0


def cpu_full_eval(threads: int) -> int:
    """One complete Omega evaluation of the benchmark workload (sweep point 5,
    M = 0.1) by the CPU oracle on `threads` host threads, timed by stage and
    checked against the committed oracle fixture of that point, beside the
    reference arm's bounded-sample estimate for the same point."""
    import numpy as np
    from oracle import oracle as orc
    from oracle.oracle import Oracle
    pts = build_points()
    n = orc.set_threads(threads)
    t0 = time.perf_counter()
    om, _, _, stages = Oracle.from_point(pts[5]).solve_timed()
    dt = time.perf_counter() - t0
    fx = float(np.load(os.path.join(ROOT, "tests", "golden", "config_c2_m05.npz"))["sft"])
    _, sample, est, wall = cpu_sample(pts[5], threads)
    print(json.dumps({"workload": WORKLOAD, "point": "M = 0.1", "cores": n, "seconds": dt,
                      "stage_seconds": {"diagonalize": stages[0], "chains": stages[1], "omega": stages[2]},
                      "omega": om, "omega_vs_fixture": abs(om - fx) / abs(fx),
                      "sample_estimate_s": est, "sample_wall_s": wall, "sample": sample}))
    return 0


def profile_mlp(steps: int) -> int:
    """Surrogate training on 200 samples of a smooth 4-input function with
    its gradient (1000 GEMM rows), `steps` Adam steps, then one prediction
    (for ncu captures of the tensor-core GEMM k_umma_gemm)."""
    import numpy as np
    from vca_gb300 import build as vbuild
    vbuild.build()
    from vca_gb300.surrogate import SurrogateNet
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (200, 4))
    w = np.array([0.7, -0.4, 0.2, 0.5])
    y = np.sin(x @ w) + 0.3 * (x ** 2).sum(axis=1)
    dy = np.cos(x @ w)[:, None] * w[None, :] + 0.6 * x
    net = SurrogateNet(n_in=4, capacity=1024, grad_weight=1.0)
    net.set_data(x, y, dy)
    t0 = time.perf_counter()
    loss = net.train(steps)
    dt = time.perf_counter() - t0
    f, df = net.predict(rng.uniform(-1, 1, (1000, 4)))
    print(json.dumps({"steps": steps, "train_s": dt, "ms_per_step": 1e3 * dt / max(1, steps), "loss": loss}))
    net.close()
    return 0


def chain_streams_ab(reps: int) -> dict:
    """The benchmark solve (point M = 0.1) with the chains' column groups one
    after another (1 stream) and two at a time (2 streams): seconds per
    solve, the chain stage, and whether Omega agrees bit for bit."""
    from vca_gb300.solver import VcaSolver
    pt = build_points()[5]
    out = {"workload": WORKLOAD, "point": "M = 0.1", "reps": reps}
    oms = []
    for n in (1, 2, 1, 2):
        cfg = pt.cfg.copy()
        cfg.hxv_variant = 2
        s = VcaSolver(cfg)
        s.set_chain_streams(n)
        s.upload_hk(pt.Hk)
        s.solve_resident(pt.Hloc)
        t0 = time.perf_counter()
        for _ in range(reps):
            om = s.solve_resident(pt.Hloc)
        dt = (time.perf_counter() - t0) / reps
        st = s.timings()
        s.close()
        oms.append(om)
        out.setdefault(f"streams_{n}", []).append({"s_per_solve": round(dt, 4), "chains_s": round(st[2] / 1e3, 4)})
    out["omega_bit_identical"] = len(set(oms)) == 1
    return out


def profile_solve() -> int:
    """One warm-up and one timed plain solve of a reduced 4x3 point."""
    from vca_gb300 import build as vbuild, clusters
    vbuild.build()
    from vca_gb300.solver import VcaSolver
    pt = clusters.square(nx=4, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=200,
                         omega_nodes=1024)
    s = VcaSolver(pt.cfg)
    s.solve(pt.Hloc, pt.Hk)
    t0 = time.perf_counter()
    om = s.solve(pt.Hloc, pt.Hk)
    print(json.dumps({"omega": om, "s": time.perf_counter() - t0, "stage_ms": s.timings().tolist(),
                      "launches": s.kernel_launches()}))
    s.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile-hxv", type=int, default=0, metavar="NCOLS",
                    help="profiling mode: load the 4x3 Hamiltonian and launch the batched H x v "
                         "on sector (7,6) with NCOLS real columns --reps times (no solve)")
    ap.add_argument("--profile-solve", action="store_true",
                    help="profiling mode: one plain solve of a reduced 4x3 point "
                         "(8x8 k-grid, 1024 nodes) after one warm-up solve")
    ap.add_argument("--profile-hxv1", action="store_true",
                    help="profiling mode: single-vector H x v on sector (8,8) of the 4x4 cluster")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--batch-c3", type=int, default=32, help="points of the C3 batch timed in the batched block")
    ap.add_argument("--batch-c4", type=int, default=256, help="points of the C4 batch timed in the batched block")
    ap.add_argument("--batched-only", action="store_true", help="only the batched block (C3 and C4)")
    ap.add_argument("--profile-batch", choices=["c3", "c4"], default=None,
                    help="profiling mode: batched form on --points points of the C3/C4 batch, then a plain solve")
    ap.add_argument("--points", type=int, default=4)
    ap.add_argument("--profile-mlp", type=int, default=0, metavar="STEPS",
                    help="profiling mode: STEPS Adam steps of the surrogate on 200 samples with gradients")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-hop-pairing", action="store_true",
                    help="--profile-hxv with the chains' kernel's plain hop order")
    ap.add_argument("--profile-hxv-c5", type=int, default=0, metavar="NCOLS",
                    help="time a NCOLS-column H x v on a chain sector of the 4x4 cluster, both forms")
    ap.add_argument("--chain-streams-ab", action="store_true",
                    help="the benchmark solve with one and with two chain streams, --reps solves each")
    ap.add_argument("--c5-solve", action="store_true",
                    help="one plain solve of the 4x4 cluster (C5), timed by stage")
    ap.add_argument("--c5-steps", type=int, default=200, help="chain steps of --c5-solve")
    ap.add_argument("--cpu-full-eval", action="store_true",
                    help="one complete oracle Omega evaluation of the benchmark workload on all host threads")
    ap.add_argument("--hxv-variant", type=int, default=2,
                    help="0 staged form, 1 warp form, 2 the chains' layout and kernel (default)")
    args = ap.parse_args()
    if args.profile_hxv:
        return profile_hxv(args.profile_hxv, args.reps, args.hxv_variant, not args.no_hop_pairing)
    if args.profile_solve:
        return profile_solve()
    if args.profile_hxv1:
        from vca_gb300 import build as vbuild
        vbuild.build()
        print(json.dumps(hxv_single_4x4(args.reps)))
        return 0
    if args.chain_streams_ab:
        from vca_gb300 import build as vbuild
        vbuild.build()
        print(json.dumps(chain_streams_ab(args.reps)))
        return 0
    if args.profile_hxv_c5:
        from vca_gb300 import build as vbuild
        vbuild.build()
        print(json.dumps(hxv_cols_4x4(args.profile_hxv_c5, args.reps)))
        return 0
    if args.c5_solve:
        from vca_gb300 import build as vbuild
        vbuild.build()
        print(json.dumps(c5_solve(args.c5_steps)))
        return 0
    if args.cpu_full_eval:
        return cpu_full_eval(os.cpu_count() or 1)
    if args.profile_mlp:
        return profile_mlp(args.profile_mlp)
    if args.profile_batch:
        return profile_batch(args.profile_batch, args.points, not args.no_autotune)
    if args.batched_only:
        from vca_gb300 import build as vbuild
        vbuild.build()
        print(json.dumps({"batched_c3": batched_block("c3", args.batch_c3, 8, 3),
                          "batched_c4": batched_block("c4", args.batch_c4, 8, 3),
                          "surrogate_search": search_block()}))
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
