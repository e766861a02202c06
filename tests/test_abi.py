"""C-ABI library checks that need no GPU: it loads, exports every symbol
declared in include/vca_gpu.h, and its config defaults match the Python
mirror of VCA_INPUT_VARS.f90 defaults."""
import ctypes
import os
import re

import pytest

from vca_gb300 import solver
from vca_gb300.config import VcaConfig, default_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "vca_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int64_t|int|void)\s+(vca_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from vca_gb300 import build
    build.build()
    return solver.load()


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(solver.EXPORTS) == syms


def test_config_layout_and_defaults(lib):
    c = solver.library_defaults()
    d = default_config()
    assert ctypes.sizeof(VcaConfig) == ctypes.sizeof(c)
    assert c.as_dict() == d.as_dict()


def test_init_without_gpu_reports_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    c = default_config(Nlat=2)
    rc = lib.vca_gpu_init(ctypes.byref(c), None, None)
    assert rc == -4
    buf = ctypes.create_string_buffer(256)
    lib.vca_gpu_last_error(buf, 256)
    assert b"no CPU fallback" in buf.value


def test_bad_config_rejected_on_host(lib):
    c = default_config(Nlat=2, Nspin=3)
    assert lib.vca_gpu_init(ctypes.byref(c), None, None) == -1
    c = default_config(Nlat=2, vca_twin=1)
    assert lib.vca_gpu_init(ctypes.byref(c), None, None) == -6
    c = default_config(Nlat=2, lanc_nstates_total=2, cutoff=0.0)
    assert lib.vca_gpu_init(ctypes.byref(c), None, None) == -1
    c = default_config(Nlat=2, lanc_nstates_total=2, lanc_niter_spectrum=0)
    assert lib.vca_gpu_init(ctypes.byref(c), None, None) == -1


def test_file_calls_without_context(lib):
    """The output-file entry points fail with VCA_ERR_STATE before a context
    exists, and the host codec checks its arguments; no GPU call is made."""
    lib.vca_gpu_finalize()
    for f in (lib.vca_gpu_print_impSigma, lib.vca_gpu_print_impG, lib.vca_gpu_print_impG0):
        assert f() == -3
    assert lib.vca_gpu_save_gfprime(b"gfprime", None, 0, 0) == -3
    assert lib.vca_gpu_read_gfprime(b"gfprime", None, 0, 0) == -3
    assert lib.vca_gfm_read(b"x", 0, 1, None, None, None, None, None, None) == -9
    assert lib.vca_gfm_write(None, 0, 0, None, None, None, None, None) == -9
    neg = (ctypes.c_int32 * 1)(-1)
    assert lib.vca_gfm_write(b"x", 0, 1, neg, None, None, None, None) == -9


def test_unterminated_file_suffix_rejected(lib):
    c = default_config(Nlat=2)
    c.file_suffix = b"x" * 64
    assert lib.vca_gpu_init(ctypes.byref(c), None, None) == -1
    assert default_config(file_suffix="_a").file_suffix == b"_a"


def test_module_names_of_the_reference(lib):
    """The public names of module VCA (VCA.f90:1-38) exist at module level in
    the Python mirror and raise VCA_ERR_STATE before vca_init_solver."""
    names = ["vca_init_solver", "vca_solve", "vca_get_sft_potential", "vca_gf_cluster", "vca_get_sigma_matsubara",
             "vca_get_sigma_realaxis", "vca_get_gimp_matsubara", "vca_get_gimp_realaxis", "vca_get_dens",
             "vca_get_mag", "vca_get_docc", "init_custom_observables", "add_custom_observable",
             "get_custom_observables", "clear_custom_observables", "vca_print_impSigma", "vca_print_impG",
             "vca_print_impG0", "save_gfprime", "read_gfprime", "vca_get_cluster_dimension",
             "search_chemical_potential", "vca_search_variable", "vca_read_impSigma", "observables_cluster"]
    for n in names:
        assert callable(getattr(solver, n)), n
    solver._solver = None
    for n in ("vca_get_dens", "vca_get_sigma_matsubara", "vca_print_impG", "get_custom_observables"):
        with pytest.raises(solver.VcaError) as e:
            getattr(solver, n)()
        assert e.value.code == -3


@pytest.mark.parametrize("cname", ["vca_config", "vca_thermal"])
def test_config_layout_matches_the_c_header(tmp_path, cname):
    """sizeof and every field offset of the C-ABI structs as a C compiler lays
    out include/vca_gpu.h equal the Python mirror's ctypes layouts; the
    header is also plain C99."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    S = VcaConfig if cname == "vca_config" else solver.VcaThermal
    names = [n for n, _ in S._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "vca_gpu.h"', "int main(void) {",
           f'  printf("%zu\\n", sizeof({cname}));']
    src += [f'  printf("%zu\\n", offsetof({cname}, {n}));' for n in names]
    src += ["  return 0;", "}"]
    (tmp_path / "layout.c").write_text("\n".join(src) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-Wall", "-I", os.path.join(ROOT, "include"), str(tmp_path / "layout.c"),
                           "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got[0] == ctypes.sizeof(S)
    assert got[1:] == [getattr(S, n).offset for n in names]
