"""GFmatrix restart files (save_gfprime / read_gfprime, VCA_AUX_FUNX.f90:
486-697): the library's host codec against the numpy restatement in
oracle/gfmatrix.py.  No GPU: the codec calls need no context.

* unformatted: the library writes the restatement's bytes exactly, and reads
  them back bit-exact;
* formatted: bit-exact round trips both ways (17 significant digits), the
  library reading the restatement's gfortran-like text with the \\n token
  after every state, and the list-directed forms a Fortran writer may use
  (values split over lines, commas, D exponents, repeat counts);
* the oracle's own tables after a solve, at T=0 and with two states;
* malformed files rejected with VCA_ERR_IO.
"""
import numpy as np
import pytest

from vca_gb300 import clusters
from vca_gb300.solver import VcaError, gfm_elements, gfprime_path, read_gfmatrix, write_gfmatrix
from oracle import gfmatrix as ogm
from oracle.oracle import Oracle

ERR_IO = -10

SPECIAL = [0.0, -0.0, 1e-300, 5e-324, -2.2250738585072014e-308, 1e300, np.pi, -1.0 / 3.0]


def random_table(seed, nelem=7):
    rng = np.random.default_rng(seed)
    table = []
    for e in range(nelem):
        el = []
        for _ in range(int(rng.integers(0, 4))):
            st = []
            for _ in range(int(rng.integers(0, 5))):
                n = int(rng.integers(0, 8))
                p = rng.normal(size=n) * 10.0 ** rng.integers(-3, 4, size=n) + 1j * rng.normal(size=n) * (e % 2)
                w = rng.normal(size=n) + 1j * rng.normal(size=n)
                if n:
                    p[0] = complex(SPECIAL[e % len(SPECIAL)], SPECIAL[(e + 3) % len(SPECIAL)])
                st.append((p, w))
            el.append(st)
        table.append(el)
    return table


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_unformatted_bytes_are_the_restatement(tmp_path, seed):
    t = random_table(seed)
    f = str(tmp_path / "g.restart")
    write_gfmatrix(f, t, formatted=False)
    ref = ogm.encode_unformatted(t)
    assert open(f, "rb").read() == ref
    assert ogm.bit_equal(read_gfmatrix(f, len(t), False), t)
    assert ogm.bit_equal(ogm.decode_unformatted(ref, len(t)), t)


@pytest.mark.parametrize("seed", [4, 5, 6])
def test_formatted_round_trips_bit_exact(tmp_path, seed):
    t = random_table(seed)
    f = str(tmp_path / "g.restart")
    write_gfmatrix(f, t, formatted=True)
    assert ogm.bit_equal(read_gfmatrix(f, len(t), True), t)
    assert ogm.bit_equal(ogm.decode_formatted(open(f).read(), len(t)), t)
    # text in gfortran's look, with \n after every state
    g = tmp_path / "h.restart"
    g.write_text(ogm.encode_formatted(t))
    assert ogm.bit_equal(read_gfmatrix(str(g), len(t), True), t)


def test_formatted_reader_accepts_list_directed_forms(tmp_path):
    text = (
        " 2\n"                                   # element 1: two states split over lines
        "  2 1 (1.5D0, -2d-1)\n"
        "(0.25 ,\n 0.75) , 0 \\n 1\n"
        "   3 3*(0,1) 2*( 1E1,0 ) (2,2)\n"
        " 1 1 2 2*(0,0) (1,0) (0,-1) \\n trailing items of the record are skipped 7 (9,9)\n"
        " 0\n"
    )
    f = tmp_path / "x.restart"
    f.write_text(text)
    t = read_gfmatrix(str(f), 3, True)
    assert len(t) == 3 and [len(e) for e in t] == [2, 1, 0]
    (p, w), (p2, w2) = t[0][0]
    np.testing.assert_array_equal(p, [1.5 - 0.2j])
    np.testing.assert_array_equal(w, [0.25 + 0.75j])
    assert len(p2) == 0 and len(w2) == 0
    (p, w), = t[0][1]
    np.testing.assert_array_equal(p, [1j, 1j, 1j])
    np.testing.assert_array_equal(w, [10, 10, 2 + 2j])
    (p, w), = t[1][0]
    np.testing.assert_array_equal(p, [0, 0])
    np.testing.assert_array_equal(w, [1, -1j])


@pytest.mark.parametrize("formatted", [False, True])
def test_oracle_tables_round_trip(tmp_path, formatted):
    pts = [
        clusters.chain1d(tprime=0.9, nlat=4, U=4.0, xmu=2.0, nk=8, ngfiter=30, omega_nodes=64),
        clusters.square(nx=2, ny=2, U=8.0, xmu=4.0, maf=0.2, nspin=2, nkx=4, nky=4, ngfiter=20,
                        omega_nodes=64),
    ]
    # two states in the list: the Hubbard atom at finite T (sectors (1,0), (0,1))
    atom = clusters.chain1d(tprime=0.0, t=0.0, nlat=1, U=4.0, xmu=2.0, nk=4, ngfiter=8, omega_nodes=64,
                            lanc_nstates_total=2, beta=20.0, bandwidth=0.0)
    pts.append(atom)
    for pt in pts:
        o = Oracle.from_point(pt)
        o.solve()
        t = ogm.table_from_oracle(o, pt.cfg)
        nel = len(gfm_elements(pt.cfg))
        assert len(t) == nel == pt.cfg.Nlat ** 2 * pt.cfg.Nspin * pt.cfg.Norb ** 2
        assert all(len(st) == (2 if (il == jl and io == jo) else 4)
                   for el, (il, jl, s, io, jo) in zip(t, gfm_elements(pt.cfg)) for st in el)
        f = str(tmp_path / "o")
        write_gfmatrix(f, t, formatted)
        assert ogm.bit_equal(read_gfmatrix(f, nel, formatted), t)
    assert [len(e) for e in t] == [2]  # the atom: one element, two states


def test_file_names():
    assert gfprime_path() == "gfprime.restart"
    assert gfprime_path("g", used=True, suffix="_x") == "g_x.used"


@pytest.mark.parametrize("formatted,data", [
    (False, b""),                                            # no record
    (False, b"\x08\x00\x00\x00\x01\x00\x00\x00"),            # truncated record
    (False, b"\x04\x00\x00\x00\x00\x00\x00\x00\x05\x00\x00\x00"),  # markers differ
    (False, b"\xfc\xff\xff\xff\x00\x00\x00\x00\xfc\xff\xff\xff"),  # continued record
    (False, b"\x04\x00\x00\x00\xff\xff\xff\xff\x04\x00\x00\x00"),  # negative count
    (False, b"\x0c\x00\x00\x00\x01\x00\x00\x00\x01\x00\x00\x00\x05\x00\x00\x00\x0c\x00\x00\x00"),  # Nexc past the record
    (True, b""),
    (True, b" 1 2 3 (1,0)\n"),                               # runs out of values
    (True, b" 1 ,, 2\n"),                                    # null value
    (True, b" 1 1 1 (1,0) oops\n"),                          # not a complex value
    (True, b" -1\n"),                                        # negative count
    (True, b" 1 1 1 (1 0) (1,0)\n"),                         # missing comma
])
def test_malformed_files_are_rejected(tmp_path, formatted, data):
    f = tmp_path / "bad.restart"
    f.write_bytes(data)
    with pytest.raises(VcaError) as e:
        read_gfmatrix(str(f), 1, formatted)
    assert e.value.code == ERR_IO


def test_missing_file_and_short_file(tmp_path):
    with pytest.raises(VcaError) as e:
        read_gfmatrix(str(tmp_path / "absent.restart"), 1, False)
    assert e.value.code == ERR_IO
    t = random_table(9, nelem=3)
    f = str(tmp_path / "three")
    write_gfmatrix(f, t, False)
    with pytest.raises(VcaError):
        read_gfmatrix(f, 4, False)  # one element more than the file holds
    assert ogm.bit_equal(read_gfmatrix(f, 2, False), t[:2])  # data after the elements read is ignored
