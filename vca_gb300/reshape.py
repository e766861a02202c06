"""The reference's index reshapes between the (Nlat,Nlat,Nspin,Nspin,Norb,
Norb) "nnn" layout and the lso matrix layout, VCA_AUX_FUNX.f90:175-468, with
is = iorb + (ilat-1)*Norb + (ispin-1)*Norb*Nlat (1-based) and, for the
so forms, is = iorb + (ispin-1)*Norb.  Real or complex, with optional
trailing axes (a function of frequency or k), Fortran order."""
from __future__ import annotations

import numpy as np


def vca_nnn2lso_reshape(Hnnn, Nlat: int, Nspin: int, Norb: int):
    """(Nlat,Nlat,Nspin,Nspin,Norb,Norb[,...]) -> (Nlso,Nlso[,...]) (:203-227, :255-279)."""
    return vca_rectangular_n2j_reshape(Hnnn, Nlat, Nlat, Nspin, Nspin, Norb, Norb)


def vca_lso2nnn_reshape(Hlso, Nlat: int, Nspin: int, Norb: int):
    """(Nlso,Nlso[,...]) -> (Nlat,Nlat,Nspin,Nspin,Norb,Norb[,...]) (:177-201, :229-253)."""
    return vca_rectangular_j2n_reshape(Hlso, Nlat, Nlat, Nspin, Nspin, Norb, Norb)


def vca_rectangular_j2n_reshape(Hlso, Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2):
    """(Nlat*Nspin*Norb, Nlat2*Nspin2*Norb2[,...]) -> (Nlat,Nlat2,Nspin,Nspin2,Norb,Norb2[,...]) (:366-390, :418-442)."""
    a = np.asarray(Hlso)
    rest = a.shape[2:]
    b = np.reshape(a, (Norb, Nlat, Nspin, Norb2, Nlat2, Nspin2) + rest, order="F")
    return np.asfortranarray(np.transpose(b, (1, 4, 2, 5, 0, 3) + tuple(range(6, b.ndim))))


def vca_rectangular_n2j_reshape(Hnnn, Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2):
    """(Nlat,Nlat2,Nspin,Nspin2,Norb,Norb2[,...]) -> (Nlat*Nspin*Norb, Nlat2*Nspin2*Norb2[,...]) (:392-416, :444-468)."""
    a = np.asarray(Hnnn)
    if a.shape[:6] != (Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2):
        raise ValueError(f"shape {a.shape[:6]} is not {(Nlat, Nlat2, Nspin, Nspin2, Norb, Norb2)}")
    rest = a.shape[6:]
    b = np.transpose(a, (4, 0, 2, 5, 1, 3) + tuple(range(6, a.ndim)))
    return np.reshape(b, (Nlat * Nspin * Norb, Nlat2 * Nspin2 * Norb2) + rest, order="F")


def vca_so2nn_reshape(Hso, Nspin: int, Norb: int):
    """(Nspin*Norb, Nspin*Norb[,...]) -> (Nspin,Nspin,Norb,Norb[,...]) (:281-318)."""
    a = np.asarray(Hso)
    rest = a.shape[2:]
    b = np.reshape(a, (Norb, Nspin, Norb, Nspin) + rest, order="F")
    return np.asfortranarray(np.transpose(b, (1, 3, 0, 2) + tuple(range(4, b.ndim))))


def vca_nn2so_reshape(Hnn, Nspin: int, Norb: int):
    """(Nspin,Nspin,Norb,Norb[,...]) -> (Nspin*Norb, Nspin*Norb[,...]) (:320-358)."""
    a = np.asarray(Hnn)
    if a.shape[:4] != (Nspin, Nspin, Norb, Norb):
        raise ValueError(f"shape {a.shape[:4]} is not {(Nspin, Nspin, Norb, Norb)}")
    rest = a.shape[4:]
    b = np.transpose(a, (2, 0, 3, 1) + tuple(range(4, a.ndim)))
    return np.reshape(b, (Nspin * Norb, Nspin * Norb) + rest, order="F")
