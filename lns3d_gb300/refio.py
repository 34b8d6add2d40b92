"""The reference's file formats: grid, metrics, mean flow, restart, potential
and history files, read and written from numpy arrays.

LNS3D keeps its state in Fortran unformatted sequential files: each record
is a 4-byte length, the payload and the length again (the gfortran layout;
the reference's test/2d case ships big-endian files written on an SGI and
run with ``GFORTRAN_CONVERT_UNIT=swap``, so every function takes an
``endian`` of "<" or ">").  Arrays are column-major with the reference's
shapes (``v(ndof, nx, ny)``, metrics ``(nx, ny)``).

* ``grid.dat`` (src/gengrid.f90:19-31, written by util/genmesh.f90:149-153):
  record 1 ``nx, ny, nz`` (int32); record 2 ``x, y, z`` for each of the nz
  planes (float64, nx*ny*nz each; z is read and discarded).
* ``metric.dat`` (src/gengrid.f90:76-79): one record ``m1, m2, n1, n2, m11,
  m12, m22, n11, n12, n22`` (float64, nx*ny each).
* ``mean.dat`` and the restart files ``output.R.N`` (src/genmean.f90:28-32,
  src/genini.f90:30-58, src/impdrv.f90:430-442): record 1 ``lstep`` (int32),
  ``time`` (float64), ``nx, ny, nz, ndof`` (int32), ``Re, Ma, Pr, gamma, cv``
  (float64), 68 bytes; record 2 the field (float64, or complex128 for the
  single-mode runs); record 3 ``vold`` when impl = 2.
* ``top.pot``, ``left.pot``, ``right.pot`` (src/potential.f90:20-60): text,
  one line ``rho u v w T`` per boundary point, read list-directed.
"""
import struct

import numpy as np

HEADER = "i d 4i 5d"


def _fmt(endian, spec):
    return endian + spec.replace(" ", "")


def write_records(path, records, endian="<"):
    """Write a sequential unformatted file: a list of bytes objects."""
    with open(path, "wb") as f:
        for rec in records:
            n = struct.pack(endian + "i", len(rec))
            f.write(n)
            f.write(rec)
            f.write(n)


def read_records(path, endian="<"):
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from(endian + "i", data, pos)
        rec = data[pos + 4:pos + 4 + n]
        (n2,) = struct.unpack_from(endian + "i", data, pos + 4 + n)
        if n2 != n or len(rec) != n:
            raise ValueError("%s: damaged record at byte %d" % (path, pos))
        out.append(rec)
        pos += 8 + n
    return out


def _arr_bytes(a, endian, dtype):
    a = np.asarray(a, dtype=dtype)
    return np.asfortranarray(a).astype(np.dtype(dtype).newbyteorder(endian)).tobytes(order="F")


def write_grid(path, x, y, endian="<", nz=1):
    x = np.asarray(x, dtype=np.float64)
    nx, ny = x.shape
    rec1 = struct.pack(endian + "3i", nx, ny, nz)
    planes = b"".join(_arr_bytes(x, endian, np.float64) for _ in range(nz))
    planes += b"".join(_arr_bytes(y, endian, np.float64) for _ in range(nz))
    planes += b"".join(_arr_bytes(np.zeros_like(x), endian, np.float64) for _ in range(nz))
    write_records(path, [rec1, planes], endian)


def read_grid(path, endian="<"):
    r = read_records(path, endian)
    nx, ny, nz = struct.unpack(endian + "3i", r[0])
    a = np.frombuffer(r[1], dtype=np.dtype(np.float64).newbyteorder(endian)).astype(np.float64)
    n = nx * ny
    x = a[:n].reshape((nx, ny), order="F").copy(order="F")
    y = a[n * nz:n * nz + n].reshape((nx, ny), order="F").copy(order="F")
    return x, y


METRIC_NAMES = ("m1", "m2", "n1", "n2", "m11", "m12", "m22", "n11", "n12", "n22")


def write_metrics(path, metrics, endian="<"):
    write_records(path, [b"".join(_arr_bytes(metrics[k], endian, np.float64) for k in METRIC_NAMES)], endian)


def read_metrics(path, nx, ny, endian="<"):
    r = read_records(path, endian)
    a = np.frombuffer(r[0], dtype=np.dtype(np.float64).newbyteorder(endian)).astype(np.float64)
    n = nx * ny
    return {k: a[i * n:(i + 1) * n].reshape((nx, ny), order="F").copy(order="F")
            for i, k in enumerate(METRIC_NAMES)}


def write_field(path, v, lstep=0, time=0.0, Re=0.0, Ma=0.0, Pr=0.0, gamma=1.4, cv=716.5, vold=None,
                endian="<", nz=1):
    """A mean-flow or restart file: the 68-byte header and the field (and vold)."""
    ndof, nx, ny = v.shape
    hdr = struct.pack(_fmt(endian, HEADER), lstep, time, nx, ny, nz, ndof, Re, Ma, Pr, gamma, cv)
    dt = np.complex128 if np.iscomplexobj(v) else np.float64
    recs = [hdr, _arr_bytes(v, endian, dt)]
    if vold is not None:
        recs.append(_arr_bytes(vold, endian, dt))
    write_records(path, recs, endian)


def read_field(path, complex_=False, endian="<"):
    """(header dict, v, vold or None)."""
    r = read_records(path, endian)
    vals = struct.unpack(_fmt(endian, HEADER), r[0])
    hdr = dict(zip(("lstep", "time", "nx", "ny", "nz", "ndof", "Re", "Ma", "Pr", "gamma", "cv"), vals))
    dt = np.dtype(np.complex128 if complex_ else np.float64).newbyteorder(endian)
    shape = (hdr["ndof"], hdr["nx"], hdr["ny"])

    def field(b):
        return np.frombuffer(b, dtype=dt).astype(dt.newbyteorder("=")).reshape(shape, order="F").copy(order="F")

    return hdr, field(r[1]), (field(r[2]) if len(r) > 2 else None)


def write_pot(path, rows):
    """rows: (n, 5) rho, u, v, w, T per boundary point."""
    with open(path, "w") as f:
        for r in np.asarray(rows, dtype=np.float64):
            f.write(" ".join("%.17e" % x for x in r) + "\n")


def read_pot(path):
    return np.loadtxt(path, dtype=np.float64, ndmin=2)


def read_history(path):
    """Numeric columns of a history file written at full precision."""
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if parts:
                rows.append([float(p) for p in parts])
    return rows


DECK_FIELDS = (
    ("Ma",), ("mattyp",), ("Re",), ("Pref", "Tref"), ("Pr",), ("dtmax", "cflmax"), ("nstep",),
    ("optx", "opty"), ("xper", "yper"), ("itout", "ntout"), ("ires",), ("ispg",), ("linear",),
    ("impl", "iLHS", "niter", "loctime"), ("top", "wall", "left", "right", "wallt"), ("eps_e", "ibuff"),
    ("omega", "x0"), ("idamp",), ("As", "Ns", "xs", "xt"), ("As2", "Ns2", "xs2", "xt2"), ("extrap",),
    ("theta",), ("tflag", "fflag", "sflag"), ("Lz",),
)

DECK_DEFAULTS = dict(Ma=0.5, mattyp=0, Re=1000.0, Pref=0.0, Tref=0.0, Pr=0.72, dtmax=1e30, cflmax=1.0, nstep=1,
                     optx=-1, opty=-1, xper=True, yper=False, itout=1, ntout=1000000, ires=1, ispg=0,
                     linear=0, impl=1, iLHS=1, niter=1, loctime=0, top=0, wall=0, left=-1, right=-1,
                     wallt=1, eps_e=0.0, ibuff=0, omega=0.0, x0=0.0, idamp=0, As=0.0, Ns=3, xs=0.8,
                     xt=1.0, As2=0.0, Ns2=3, xs2=0.8, xt2=1.0, extrap=-1, theta=0.0, tflag=False,
                     fflag=False, sflag=False, Lz=0.0)


def _deck_val(v):
    if isinstance(v, bool):
        return ".true." if v else ".false."
    if isinstance(v, (int, np.integer)):
        return "%d" % v
    return repr(float(v))


def write_deck(values):
    """The positional input deck read by src/input.f90:14-302 (one line per read)."""
    d = dict(DECK_DEFAULTS)
    d.update(values)
    lines = []
    for fields in DECK_FIELDS:
        lines.append(" ".join(_deck_val(d[f]) for f in fields) + "    ! " + ", ".join(fields))
    return "\n".join(lines) + "\n"


def parse_deck(text):
    """Values of a positional deck, read list-directed as src/input.f90 does."""
    tokens_per_line = []
    for line in text.splitlines():
        toks = line.replace(",", " ").split()
        tokens_per_line.append(toks)
    out = {}
    li = 0
    for fields in DECK_FIELDS:
        toks = []
        while len(toks) < len(fields):
            toks += tokens_per_line[li]
            li += 1
        for f, t in zip(fields, toks):
            ref = DECK_DEFAULTS[f]
            if isinstance(ref, bool):
                out[f] = t.strip(".").lower().startswith("t")
            elif isinstance(ref, int):
                out[f] = int(t)
            else:
                out[f] = float(t.lower().replace("d", "e"))
    return out
