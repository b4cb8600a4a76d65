"""Writers of the reference's binary hand-off files for the tests, with the
layouts of the psi4 plugin's writers (syshfwplug/plugin.cc:251-257, 328-333,
518-520, 558-571, 636-652), except that the three basis names are written as
NUL-padded 32-byte fields, the layout read_system reads (src/IO/ops_io.cc:97-99)."""
import numpy as np


def write_sys(prefix, nroe, nroao, naux_1, naux_2, nrofint, nrofaux, nrofaux2, coord, charges,
              zeff, mass, names):
    with open(prefix + ".sys", "wb") as f:
        f.write(np.array([nroe, len(charges), nroao, naux_1, naux_2], dtype=np.int32).tobytes())
        f.write(np.array([nrofint, nrofaux, nrofaux2], dtype=np.int64).tobytes())
        for a in (coord, charges, zeff, mass):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for n in names:
            f.write(n.encode().ljust(32, b"\0"))


def write_oei(prefix, H, T, S, V):
    with open(prefix + ".oei", "wb") as f:
        for a in (H, T, S, V):
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


def write_tei(prefix, sortcount, intval, intnums):
    with open(prefix + ".tei", "wb") as f:
        f.write(np.asarray(sortcount, dtype=np.int64).tobytes())
        f.write(np.ascontiguousarray(intval, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(intnums, dtype=np.uint16).tobytes())


def write_rimp2(prefix, bpq):
    with open(prefix + ".rimp2", "wb") as f:
        f.write(np.ascontiguousarray(bpq, dtype=np.float64).tobytes())


def random_system(r, na):
    coord = r.standard_normal((na, 3))
    charges = r.integers(1, 9, na).astype(np.float64)
    return coord, charges, charges.copy(), 1.5 * charges
