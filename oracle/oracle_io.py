"""CPU oracle of the reference's solution / restart files -- TEST
INFRASTRUCTURE ONLY.  Tests use it to check the library's files byte for
byte; nothing in the package imports it.

Restates, with numpy on the host:
  astore       src/io.f:2-170     file names, mesh-count / size records,
                                  store per mesh, turbulence files, istep0
  store        src/io.f:278-340   q(1:4)*J record (in place, then /J again),
                                  q(5:nv) record, grid record x, y (+iblank)
  storevnu     src/io.f:173-215   Tecplot zone of x, y, iblank, q(5)
  storekomega  src/io.f:218-275   q(5:nv) record again, Tecplot zone of
                                  x, y, iblank, q(5)/rho, q(6)/rho
  restr2, restr_turb, qdivj       src/io.f:383-425, src/init.f:138-206

Record framing: Fortran sequential unformatted records as gfortran and ifort
write them below 2 GiB (int32 byte count, payload, int32 byte count), reals
8 bytes (the reference is built with -r8), integers 4 bytes.  The framing is
pinned against scipy.io.FortranFile, an independent reader of that format;
no Fortran compiler exists here to run the reference's own io.f, so the
byte layout beyond the framing is unpinned.

Formatted output: '(3F22.13)' and '(3I10)' as written; list-directed lines
(" ZONE", " I = ...") in gfortran's layout (leading blank, integers in 12
columns).
"""
import math
import os
import struct

import numpy as np


# ---------------------------------------------------------------- records

def rec_bytes(*parts):
    """One unformatted record of the concatenated parts (numpy arrays, taken
    in Fortran element order, or bytes)."""
    payload = b"".join(p if isinstance(p, (bytes, bytearray)) else np.asarray(p).tobytes(order="F")
                       for p in parts)
    m = struct.pack("<i", len(payload))
    return m + payload + m


def read_records(path):
    """All records of an unformatted sequential file, as bytes."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    i = 0
    while i < len(data):
        (m,) = struct.unpack_from("<i", data, i)
        out.append(data[i + 4:i + 4 + m])
        (m2,) = struct.unpack_from("<i", data, i + 4 + m)
        assert m2 == m, "record markers differ"
        i += 8 + m
    return out


# ---------------------------------------------------------- formatted text

def fmt_f(v, w=22, d=13):
    if math.isnan(v):
        s = "NaN".rjust(w)
    elif math.isinf(v):
        s = ("Infinity" if v > 0 else "-Infinity").rjust(w)
    else:
        s = "%*.*f" % (w, d, v)
    return "*" * w if len(s) > w else s


def tec_reals(vals):
    vals = np.asarray(vals, dtype=np.float64).ravel(order="F")
    if vals.size == 0:
        return "\n"
    lines = []
    for i in range(0, vals.size, 3):
        lines.append("".join(fmt_f(float(v)) for v in vals[i:i + 3]) + "\n")
    return "".join(lines)


def tec_ints(vals):
    vals = np.asarray(vals).ravel(order="F")
    if vals.size == 0:
        return "\n"
    lines = []
    for i in range(0, vals.size, 3):
        lines.append("".join(("%10d" % int(v)) if len("%10d" % int(v)) <= 10 else "*" * 10
                             for v in vals[i:i + 3]) + "\n")
    return "".join(lines)


def tec_title(iturb):
    t = ' TITLE = "Turbulence Model solution File"\n'
    if iturb == 2:
        return t + ' VARIABLES = "X" "Y" "IBlank" "K" "Omega"\n'
    return t + ' VARIABLES = "X" "Y" "IBlank" "Vnu_t"\n'


def tec_zone(jd, kd):
    return " ZONE\n I = %12d, J = %12d\n ZONETYPE = Ordered, DATAPACKING = BLOCK\n" % (jd, kd)


# ------------------------------------------------------------------ names

def sol_file(d, ts, nsp, kind, iturb):
    """astore's file names (io.f:39-53, :87-95, :123-131) and init.f:141-148."""
    n = str(nsp)
    if kind == "g":
        name = "fort_TS%s.9" % n if ts else "fort.9"
    elif kind == "q":
        name = "fort_TS%s.8" % n if ts else "fort.8"
    elif kind == "r":
        name = "fort_TS%s.3" % n if ts else "fort.3"
    else:
        base = "komega" if iturb == 2 else "SA"
        name = (base + "_TS" + n if ts else base) + ".dat"
    return os.path.join(d, name)


# ------------------------------------------------------------------ astore

def _q4(q, jd, kd, nspec, nq):
    return q.reshape((jd, kd, nspec, nq), order="F")


def astore(d, p, meshes, istep0, ts):
    """io.f:2-170.  p: object with fsmach, alfa, rey (rey/fsmach as
    read_inputs keeps it), totime, iturb, itrans, nspec, nq, nv.  meshes: list
    of dicts with q (flat, modified in place by store's round trip), x, y,
    iblank (flat (jd,kd,nspec)), jd, kd.  Writes the files into d."""
    assert p.itrans == 0
    nm, ns, it = len(meshes), p.nspec, p.iturb
    turb = it in (1, 2)
    dims = np.array([v for m in meshes for v in (m["jd"], m["kd"])], dtype=np.int32)
    fg = [bytearray() for _ in range(ns)]
    fq = [bytearray() for _ in range(ns)]
    ft = ["" for _ in range(ns)]
    for s in range(ns):
        for b in (fg[s], fq[s]):
            if nm > 1:
                b += rec_bytes(np.array([nm], dtype=np.int32))
            b += rec_bytes(dims)
    hdr = np.array([p.fsmach, p.alfa, p.rey * p.fsmach, p.totime], dtype=np.float64)
    for m in meshes:   # store, io.f:278-340
        jd, kd = m["jd"], m["kd"]
        q = _q4(m["q"], jd, kd, ns, p.nq)
        x = m["x"].reshape((jd, kd, ns), order="F")
        y = m["y"].reshape((jd, kd, ns), order="F")
        ib = m["iblank"].reshape((jd, kd, ns), order="F")
        for s in range(ns):
            J = q[:, :, s, p.nq - 1].copy()
            for n in range(4):
                q[:, :, s, n] = q[:, :, s, n] * J
            fq[s] += rec_bytes(hdr)
            fq[s] += rec_bytes(np.asfortranarray(q[:, :, s, 0:4]))
            if turb:
                fq[s] += rec_bytes(np.asfortranarray(q[:, :, s, 4:p.nv]))
            parts = [np.asfortranarray(x[:, :, s]), np.asfortranarray(y[:, :, s])]
            if nm > 1:
                parts.append(np.asfortranarray(ib[:, :, s]).astype(np.int32))
            fg[s] += rec_bytes(*parts)
            for n in range(4):   # qdivj, io.f:332
                q[:, :, s, n] = q[:, :, s, n] / J
    if turb:
        for s in range(ns):
            ft[s] += tec_title(it)
        for m in meshes:   # storevnu / storekomega
            jd, kd = m["jd"], m["kd"]
            q = _q4(m["q"], jd, kd, ns, p.nq)
            x = m["x"].reshape((jd, kd, ns), order="F")
            y = m["y"].reshape((jd, kd, ns), order="F")
            ib = m["iblank"].reshape((jd, kd, ns), order="F")
            for s in range(ns):
                if it == 2:
                    rho = q[:, :, s, 0] * q[:, :, s, p.nq - 1]
                    fq[s] += rec_bytes(np.asfortranarray(q[:, :, s, 4:p.nv]))
                ft[s] += tec_zone(jd, kd)
                ft[s] += tec_reals(x[:, :, s]) + tec_reals(y[:, :, s]) + tec_ints(ib[:, :, s])
                if it == 1:
                    ft[s] += tec_reals(q[:, :, s, 4])
                else:
                    ft[s] += tec_reals(q[:, :, s, 4] / rho) + tec_reals(q[:, :, s, 5] / rho)
    for s in range(ns):
        fq[s] += rec_bytes(np.array([istep0], dtype=np.int32))
        with open(sol_file(d, ts, s + 1, "g", it), "wb") as f:
            f.write(bytes(fg[s]))
        with open(sol_file(d, ts, s + 1, "q", it), "wb") as f:
            f.write(bytes(fq[s]))
        if turb:
            with open(sol_file(d, ts, s + 1, "t", it), "w") as f:
                f.write(ft[s])


# ----------------------------------------------------------------- restart

def restart(d, p, q, jd, kd, ts):
    """init.f:138-170 for one mesh (num_grids = 1): reads fort.3 (fort_TS<n>.3)
    into q (flat (jd,kd,nspec,nq), J already in q(nq)) and divides q(1:4) by
    J.  Returns (totime, istep0)."""
    ns = p.nspec
    qq = _q4(q, jd, kd, ns, p.nq)
    turb = p.iturb in (1, 2)
    totime = istep0 = None
    for s in range(ns):
        recs = read_records(sol_file(d, ts, s + 1, "r", p.iturb))
        hdr = np.frombuffer(recs[1][:32], dtype=np.float64)
        totime = float(hdr[3])
        n2 = jd * kd
        qq[:, :, s, 0:4] = np.frombuffer(recs[2][:4 * n2 * 8], dtype=np.float64).reshape((jd, kd, 4), order="F")
        k = 3
        if turb:
            nt = p.nv - 4
            qq[:, :, s, 4:p.nv] = np.frombuffer(recs[3][:nt * n2 * 8],
                                                dtype=np.float64).reshape((jd, kd, nt), order="F")
            k = 4
        istep0 = int(np.frombuffer(recs[k][:4], dtype=np.int32)[0])
        J = qq[:, :, s, p.nq - 1].copy()
        for n in range(4):
            qq[:, :, s, n] = qq[:, :, s, n] / J
    return totime, istep0
