"""Generate the golden fixtures in tests/golden/ (run from the repo root).

The reference (Fortran + SciFortran) cannot be built in this container, so the
fixtures come from the CPU oracle and are cross-checked here, before writing,
against independent numpy computations:
  * sector ground-state energies against dense LAPACK diagonalisation of the
    sector matrices (numpy.linalg.eigvalsh);
  * Fock maps against a direct enumeration of popcount words.
Contents:
  chain4.npz   4-site Hubbard chain, U=4, xmu=2, 64 k-points, 100-step chains,
               4096-node Omega rule; t' swept over linspace(0.8, 1.2, 21):
               E_gs, Omega integral, SFT potential, sector energies at t'=1,
               G'(i w) at t'=1 on 6 frequencies.
  small_models.npz  E_gs / Omega / G'(i w) of a spin-polarised 2x2 cluster,
               a 2x2+2 bath cluster and a BHZ 2x2 cluster (complex H).
  mid_models.npz  larger sectors than the oracle runs inside the GPU tests:
               the 3x3 AFM cluster (U=8, xmu=4, M=0.1, Nspin=2, sectors up to
               15,876) at T=0 and at beta=10 (the finite-T list, zeta, Omega'
               and the two parts of the Omega integral), and a 2x2 cluster
               with 6 bath levels (sectors up to 63,504) at T=0.
  config_<name>.npz  one point of each full-size workload, at exactly the
               sizes the benchmark and the batched form run (minutes to an
               hour of oracle time each on a multi-core host):
               c2_m00 / c2_m05: the 4x3 cluster (U=8, xmu=4, Nspin=2, 32x32 k,
               200-step chains, 8192 nodes) at M = 0 and M = 0.1 (sweep
               points 0 and 5 of linspace(0, 0.3, 16));
               c3_p0: the first point of the 2x2 + 8 bath batch (24x24 k,
               200-step chains, 4096 nodes);
               c4_p0: the first point of the BHZ batch (48x48 k, 200-step
               chains, 4096 nodes).
               Each holds E_gs, the Omega integral, the SFT potential, every
               sector energy and G'(i w) at the WG frequencies.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from vca_gb300 import clusters  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
WG = np.array([0.05, 0.2, 0.7, 1.5, 4.0, 20.0])


def check_energies(o):
    for isec in range(1, o.Nsectors + 1):
        if o.dim(isec) > 2500:
            continue
        w = np.linalg.eigvalsh(o.dense_h(isec))
        assert abs(o.sector_energies()[isec - 1] - w[0]) < 1e-11 * max(1, abs(w[0])), isec


def chain4():
    tps = np.linspace(0.8, 1.2, 21)
    egs, oi, sft = [], [], []
    for tp in tps:
        pt = clusters.chain1d(tprime=float(tp), nlat=4, U=4.0, xmu=2.0, nk=64, ngfiter=100,
                              omega_nodes=4096)
        o = Oracle.from_point(pt)
        a, b, c = o.solve()
        sft.append(a)
        egs.append(b)
        oi.append(c)
        if abs(tp - 1.0) < 1e-12:
            check_energies(o)
            sec_e = o.sector_energies()
            g = o.gf_cluster(1j * WG)
    np.savez_compressed(os.path.join(OUT, "chain4.npz"), tprime=tps, egs=np.array(egs),
                        omega_int=np.array(oi), sft=np.array(sft), sector_e_t1=sec_e, wg=WG,
                        g_t1=g)


def small_models():
    out = {}
    pts = {
        "sq2x2": clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=6, nky=6, ngfiter=80,
                                 omega_nodes=1024),
        "bath": clusters.square_bath(nb=2, nk1=6, ngfiter=60, omega_nodes=1024),
        "bhz": clusters.bhz(mass=2.2, delta=0.1, nk1=4, ngfiter=60, omega_nodes=1024),
    }
    for name, pt in pts.items():
        o = Oracle.from_point(pt)
        a, b, c = o.solve()
        check_energies(o)
        out[name + "_sft"] = a
        out[name + "_egs"] = b
        out[name + "_omega_int"] = c
        out[name + "_g"] = o.gf_cluster(1j * WG)
    out["wg"] = WG
    np.savez_compressed(os.path.join(OUT, "small_models.npz"), **out)


def mid_points():
    sq = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=100,
                         omega_nodes=2048)
    ft = clusters.square(nx=3, ny=3, U=8.0, xmu=4.0, maf=0.1, nspin=2, nkx=8, nky=8, ngfiter=80,
                         omega_nodes=256)
    c = ft.cfg.copy()
    c.lanc_nstates_total, c.beta, c.bandwidth = 2, 10.0, 8.0
    ft.cfg = c
    bath = clusters.square_bath(nb=6, nk1=6, ngfiter=80, omega_nodes=1024)
    return {"sq3x3": sq, "sq3x3_b10": ft, "bath6": bath}


def mid_models():
    out = {}
    for name, pt in mid_points().items():
        o = Oracle.from_point(pt)
        a, b, c = o.solve()
        check_energies(o)
        out[name + "_sft"] = a
        out[name + "_egs"] = b
        out[name + "_omega_int"] = c
        out[name + "_sector_e"] = o.sector_energies()
        out[name + "_g"] = o.gf_cluster(1j * WG)
        if pt.cfg.lanc_nstates_total != 1:
            t = o.thermal()
            out[name + "_states"] = np.array(sorted(s for s, _ in o.states()))
            for key in ("zeta", "omega_prime", "max_exc", "sum_part", "contour_part"):
                out[name + "_" + key] = t[key]
            out[name + "_nmax"] = t["nmax"]
    out["wg"] = WG
    np.savez_compressed(os.path.join(OUT, "mid_models.npz"), **out)


def config_points():
    """The full-size points, built exactly as bench.py builds its workloads."""
    ms = np.linspace(0.0, 0.3, 16)
    c2 = {f"c2_m{i:02d}": clusters.square(nx=4, ny=3, U=8.0, xmu=4.0, maf=float(ms[i]), nspin=2, nkx=32,
                                           nky=32, ngfiter=200, omega_nodes=8192) for i in (0, 5)}
    return {
        "c4_p0": clusters.batch_bhz(B=1)[0],
        "c3_p0": clusters.batch_square_bath(B=1)[0],
        **c2,
    }


def config_models(names=None):
    for name, pt in config_points().items():
        if names and name not in names:
            continue
        o = Oracle.from_point(pt)
        a, b, c = o.solve()
        out = {"sft": a, "egs": b, "omega_int": c, "sector_e": o.sector_energies(),
               "g": o.gf_cluster(1j * WG), "wg": WG,
               "states": np.array(sorted(s for s, _ in o.states()))}
        np.savez_compressed(os.path.join(OUT, f"config_{name}.npz"), **out)
        print(name, "written", flush=True)


if __name__ == "__main__":
    # optional arguments name the fixtures to write (chain4, small, mid, configs
    # or one config point such as c3_p0); chain4, small and mid by default
    args = set(sys.argv[1:])
    if args & set(config_points()) or "configs" in args:
        config_models(None if "configs" in args else args & set(config_points()))
        sys.exit(0)
    which = args or {"chain4", "small", "mid"}
    if "chain4" in which:
        chain4()
    if "small" in which:
        small_models()
    if "mid" in which:
        mid_models()
    print("fixtures written to", OUT)
