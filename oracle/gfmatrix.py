"""GFmatrix restart-file layout restated with numpy and struct.

Test infrastructure: the oracle for the library's save_gfprime /
read_gfprime.  Nothing in the product imports it.

Follows VCA_AUX_FUNX.f90 of QcmPlab/VCA:
* the parent statements of save_gfprime / read_gfprime (:601-697) write and
  read one GFmatrix per spin-diagonal element, ilat outermost and jorb
  innermost (:627-641);
* write_unformatted / read_unformatted (:547-593): inside the element's one
  sequential record, Nstates, per state Nchan, per channel Nexc then the
  poles then the weights; records framed by their 4-byte length;
* write_formatted / read_formatted (:486-539): the same items as
  list-directed text; the writer puts the two characters \\n after every
  state (:503).

The formatted writer here imitates gfortran's list-directed look: blanks
before items, integers right-justified in 12 columns, complex numbers as
(re,im) with each part in 17 significant digits and blank padding inside the
parentheses.  The library's reader is checked on text that it did not write.

A table is a list over elements (file order) of lists over states of lists
over channels of (poles, weights) complex arrays.
"""
from __future__ import annotations

import re
import struct

import numpy as np


def elements(Nlat: int, Nspin: int, Norb: int):
    """(ilat, jlat, ispin, iorb, jorb), 1-based, in file order."""
    out = []
    for il in range(1, Nlat + 1):
        for jl in range(1, Nlat + 1):
            for s in range(1, Nspin + 1):
                for io in range(1, Norb + 1):
                    for jo in range(1, Norb + 1):
                        out.append((il, jl, s, io, jo))
    return out


def table_from_oracle(o, cfg):
    """The oracle's impGmatrix after a solve: every state of the list, the
    channels the oracle built for it (2, or 4 off the diagonal with chan4),
    each channel's poles and weights."""
    table = []
    for (il, jl, s, io, jo) in elements(cfg.Nlat, cfg.Nspin, cfg.Norb):
        el = []
        k = 0
        while o.gf_channel(il, jl, s, io, jo, k, 1) is not None:
            st = []
            ch = 1
            while True:
                r = o.gf_channel(il, jl, s, io, jo, k, ch)
                if r is None:
                    break
                st.append((r[0].copy(), r[1].copy()))
                ch += 1
            el.append(st)
            k += 1
        table.append(el)
    return table


# ---- unformatted ---------------------------------------------------------
def encode_unformatted(table) -> bytes:
    out = bytearray()
    for el in table:
        body = bytearray(struct.pack("<i", len(el)))
        for st in el:
            body += struct.pack("<i", len(st))
            for p, w in st:
                p = np.asarray(p, dtype="<c16")
                w = np.asarray(w, dtype="<c16")
                body += struct.pack("<i", len(p)) + p.tobytes() + w.tobytes()
        out += struct.pack("<i", len(body)) + body + struct.pack("<i", len(body))
    return bytes(out)


def decode_unformatted(data: bytes, nelem: int):
    table, off = [], 0
    for _ in range(nelem):
        (m,) = struct.unpack_from("<i", data, off)
        rec = data[off + 4:off + 4 + m]
        (m2,) = struct.unpack_from("<i", data, off + 4 + m)
        if m2 != m or len(rec) != m:
            raise ValueError("bad record framing")
        off += m + 8
        q = 0

        def i32():
            nonlocal q
            (v,) = struct.unpack_from("<i", rec, q)
            q += 4
            return v

        def cvec(n):
            nonlocal q
            v = np.frombuffer(rec, dtype="<c16", count=n, offset=q).astype(np.complex128)
            q += 16 * n
            return v

        el = []
        for _ in range(i32()):
            st = []
            for _ in range(i32()):
                n = i32()
                p = cvec(n)
                w = cvec(n)
                st.append((p, w))
            el.append(st)
        table.append(el)
    return table


# ---- formatted -----------------------------------------------------------
def encode_formatted(table) -> str:
    lines = []
    for el in table:
        parts = [f"{len(el):12d}"]
        for st in el:
            parts.append(f"{len(st):12d}")
            for p, w in st:
                parts.append(f"{len(p):12d}")
                for v in list(p) + list(w):
                    parts.append(f"({v.real:25.16E}     ,{v.imag:25.16E}     )")
            parts.append("\\n")
        lines.append(" " + " ".join(parts))
    return "\n".join(lines) + "\n"


_TOKEN = re.compile(r"\(\s*([^,()\s]+)\s*,\s*([^,()\s]+)\s*\)|([+-]?\d+)(?=[\s,]|$)|\\n")


def decode_formatted(text: str, nelem: int):
    """One line per element; the parts of a value may not span lines here
    (the writers on both sides put an element on one line)."""
    lines = text.split("\n")
    table = []
    for e in range(nelem):
        toks = []
        for m in _TOKEN.finditer(lines[e]):
            if m.group(1) is not None:
                toks.append(complex(float(m.group(1).replace("D", "e").replace("d", "e")),
                                    float(m.group(2).replace("D", "e").replace("d", "e"))))
            elif m.group(3) is not None:
                toks.append(int(m.group(3)))
        it = iter(toks)
        el = []
        for _ in range(next(it)):
            st = []
            for _ in range(next(it)):
                n = next(it)
                p = np.array([next(it) for _ in range(n)], dtype=np.complex128)
                w = np.array([next(it) for _ in range(n)], dtype=np.complex128)
                st.append((p, w))
            el.append(st)
        table.append(el)
    return table


def same_structure(a, b) -> bool:
    if len(a) != len(b):
        return False
    for ea, eb in zip(a, b):
        if len(ea) != len(eb):
            return False
        for sa, sb in zip(ea, eb):
            if len(sa) != len(sb):
                return False
            for (pa, wa), (pb, wb) in zip(sa, sb):
                if len(pa) != len(pb) or len(wa) != len(wb):
                    return False
    return True


def bit_equal(a, b) -> bool:
    if not same_structure(a, b):
        return False
    for ea, eb in zip(a, b):
        for sa, sb in zip(ea, eb):
            for (pa, wa), (pb, wb) in zip(sa, sb):
                if np.asarray(pa, np.complex128).tobytes() != np.asarray(pb, np.complex128).tobytes():
                    return False
                if np.asarray(wa, np.complex128).tobytes() != np.asarray(wb, np.complex128).tobytes():
                    return False
    return True
