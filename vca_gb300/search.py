"""The reference's density searches, VCA_AUX_FUNX.f90:700-897: host-side
helpers a driver calls between vca_solve calls to move xmu (or any other
variable) until the density ntmp the solve returns meets NREAD.

* search_chemical_potential (:792-897, public in module VCA): steps of
  NDELTA in the direction of the error, the step halved when the direction
  flips, the acceptance threshold lowered by a decade each time the density
  meets it in a converged outer loop;
* vca_search_variable (:709-783): a secant step on the measured
  compressibility (NDELTA as the first guess, or var_compressibility.restart).

Both are plain arithmetic on the numbers the caller passes; the Fortran SAVE
variables live in a SearchState.  As in the reference they append to
search_mu_iteration<file_suffix>.ed / search_variable_iteration_info
<file_suffix>.ed and write var_compressibility.used in the working directory
(write_files=False turns that off).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field


@dataclass
class SearchState:
    # input variables (VCA_INPUT_VARS.f90:64-67,165-167).  niter is declared
    # there but never read from the input file: a module variable that stays
    # 0 unless a driver assigns it.
    nread: float = 0.0
    nerr: float = 1e-4
    ndelta: float = 0.1
    niter: int = 0
    file_suffix: str = ""
    write_files: bool = True
    # SAVE variables of search_chemical_potential (VCA_AUX_FUNX.f90:798-804)
    count: int = 0
    totcount: int = 0
    nindex: int = 0
    nth_magnitude: int = -2
    nth_magnitude_old: int = -2
    nth: float = 1e-2
    ireduce: bool = True
    # SAVE variables of vca_search_variable (:714-721)
    v_count: int = 0
    v_totcount: int = 0
    chich: float = 0.0
    nold: float = 0.0
    var_new: float = 0.0
    var_old: float = 0.0
    log: list = field(default_factory=list)


def _append(st: SearchState, name: str, line: str, header: str | None = None):
    if not st.write_files:
        return
    with open(name, "a") as f:
        if header is not None:
            f.write(header + "\n")
        f.write(line + "\n")


def search_chemical_potential(st: SearchState, var: float, ntmp: float, converged: bool):
    """One call of search_chemical_potential(var, ntmp, converged): returns
    the new (var, converged).  st.ndelta is updated in place, as the
    reference updates its input variable NDELTA.

    The history nindex_old(3) of the reference is a local array without
    SAVE: only nindex_old(1) is assigned on every call, so entries 2 and 3
    hold whatever the stack held.  They are taken as 0 here, which leaves
    the flip test of the commented-out form at :830, a step against the
    previous call's direction."""
    ndiff = ntmp - st.nread
    nratio = 0.5
    st.count += 1
    st.totcount += 1
    nindex_old = [st.nindex, 0, 0]
    if ndiff >= st.nth:
        nindex = -1
    elif ndiff <= -st.nth:
        nindex = 1
    else:
        nindex = 0
    ndelta_old = st.ndelta
    flip = nindex != 0 and (nindex + nindex_old[0] == 0 or nindex + sum(nindex_old) == 0)
    st.ndelta = ndelta_old * nratio if flip else ndelta_old
    if ndelta_old < 1e-9:
        ndelta_old = 0.0
        nindex = 0
    st.nindex = nindex
    var = var + float(nindex) * st.ndelta
    st.log.append((var, ntmp, ndiff))
    _append(st, f"search_mu_iteration{st.file_suffix}.ed", f"{var!r} {ntmp!r} {ndiff!r}")
    # a converged outer loop inside the current threshold: lower it a decade
    if st.ireduce and abs(ndiff) < st.nth and converged and st.nth > st.nerr:
        st.nth_magnitude_old = st.nth_magnitude
        st.nth_magnitude = st.nth_magnitude_old - 1
        st.nth = max(st.nerr, 10.0 ** st.nth_magnitude)
        st.count = 0
        converged = False
        st.ndelta = ndelta_old * nratio
    if abs(ntmp - st.nread) > st.nth:
        converged = False
    # more than niter calls at this threshold without convergence: back to
    # the previous threshold, no more reductions
    if st.ireduce and st.count > st.niter and not converged:
        st.ireduce = False
        st.nth = 10.0 ** st.nth_magnitude_old
    return var, converged


def vca_search_variable(st: SearchState, var: float, ntmp: float, converged: bool):
    """One call of vca_search_variable(var, ntmp, converged): a secant step
    var - (ntmp - NREAD)/chi with chi = dn/dvar from the previous call (NDELTA,
    or the value in var_compressibility.restart, on the first).  Returns the
    new (var, converged)."""
    st.v_count += 1
    st.v_totcount += 1
    if st.v_count == 1:
        st.chich = st.ndelta
        if os.path.exists("var_compressibility.restart"):
            with open("var_compressibility.restart") as f:
                st.chich = float(f.read().split()[0].replace("D", "e").replace("d", "e"))
        st.var_old = var
    ndiff = ntmp - st.nread
    if st.v_count > 1:
        st.chich = (ntmp - st.nold) / (var - st.var_old)
    st.var_new = var - ndiff / st.chich
    st.nold = ntmp
    st.var_old = var
    var = st.var_new
    st.log.append((var, ntmp, ndiff))
    _append(st, f"search_variable_iteration_info{st.file_suffix}.ed", f"{var!r} {ntmp!r} {ndiff!r}",
            header="#var,ntmp,ndiff" if st.v_count == 1 else None)
    if abs(ndiff) > st.nerr:
        converged = False
    if st.write_files:
        with open("var_compressibility.used", "w") as f:
            f.write(f"{st.chich!r}\n")
    return var, converged
