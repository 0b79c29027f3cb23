"""Test helpers: write .re2 files (the layout core/reader_re2.f reads) for box
meshes of straight-sided hexahedra, with optional vertex perturbation,
periodic y faces, element reordering and either word size / byte order."""
import struct

import numpy as np

# preprocessor corner c (0-based) of an element -> (i, j, k) tensor offsets
PRE_CORNERS = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1),
               (0, 1, 1)]
# preprocessor faces: 1 y-, 2 x+, 3 y+, 4 x-, 5 z-, 6 z+  -> (axis, side)
PRE_FACES = {1: (1, 0), 2: (0, 1), 3: (1, 1), 4: (0, 0), 5: (2, 0), 6: (2, 1)}


def box_elements(kx, ky, kz, periodic_y=False, jitter=0.0, seed=0, perm=None):
    """Corners (nel, 8) x/y/z in preprocessor order, the lattice vertex id of
    every corner (tensor order, for checks), and boundary records
    [(element 1-based, face, values(5), type)].  Interior lattice vertices are
    moved by up to jitter * h; y-periodic meshes wrap the y lattice.  perm
    reorders the elements (file element q is box element perm[q])."""
    rng = np.random.default_rng(seed)
    nvx, nvy, nvz = kx + 1, ky + 1, kz + 1
    X, Y, Z = np.meshgrid(np.arange(nvx) / kx, np.arange(nvy) / ky, np.arange(nvz) / kz,
                          indexing="ij")
    P = np.stack([X, Y, Z], axis=-1)
    inner = np.zeros((nvx, nvy, nvz), dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    h = 1.0 / max(kx, ky, kz)
    P[inner] += jitter * h * rng.uniform(-1, 1, (int(inner.sum()), 3))
    nel = kx * ky * kz
    order = np.arange(nel) if perm is None else np.asarray(perm)
    xc, yc, zc = (np.zeros((nel, 8)) for _ in range(3))
    lattice = np.zeros((nel, 8), dtype=np.int64)
    pos = np.empty(nel, dtype=np.int64)
    pos[order] = np.arange(nel)  # box element -> file position
    for q, eb in enumerate(order):
        ex, ey, ez = eb % kx, (eb // kx) % ky, eb // (kx * ky)
        for c, (i, j, k) in enumerate(PRE_CORNERS):
            vx, vy, vz = ex + i, ey + j, ez + k
            xc[q, c], yc[q, c], zc[q, c] = P[vx, vy, vz]
        for c in range(8):  # tensor order
            i, j, k = c & 1, (c >> 1) & 1, c >> 2
            vy = (ey + j) % ky if periodic_y else ey + j
            lattice[q, c] = 1 + (ex + i) + nvx * (vy + nvy * (ez + k))
    bcs = []
    for q, eb in enumerate(order):
        ex, ey, ez = eb % kx, (eb // kx) % ky, eb // (kx * ky)
        idx = (ex, ey, ez)
        lim = (kx, ky, kz)
        for f, (ax, side) in PRE_FACES.items():
            on = idx[ax] == (lim[ax] - 1 if side else 0)
            if not on:
                continue
            if ax == 1 and periodic_y:
                ey2 = 0 if side else ky - 1
                partner = ex + kx * (ey2 + ky * ez)
                pf = 1 if side else 3
                bcs.append((q + 1, f, (float(pos[partner] + 1), float(pf), 0.0, 0.0, 0.0), "P  "))
            else:
                bcs.append((q + 1, f, (0.0,) * 5, "W  "))
    return xc, yc, zc, lattice, bcs


# proper rotations of an element's corner list (preprocessor order): a
# quarter turn about t, and a half turn about r
ROT_T = [1, 2, 3, 0, 5, 6, 7, 4]
ROT_R = [7, 6, 5, 4, 3, 2, 1, 0]


def rotate_elements(xc, yc, zc, seed=0):
    """The same hexahedra with their corner lists rotated at random (a mix of
    local frames, as in unstructured meshes)."""
    rng = np.random.default_rng(seed)
    out = [a.copy() for a in (xc, yc, zc)]
    for q in range(xc.shape[0]):
        order = list(range(8))
        for _ in range(int(rng.integers(0, 4))):
            order = [order[c] for c in ROT_T]
        if rng.integers(0, 2):
            order = [order[c] for c in ROT_R]
        for a, src in zip(out, (xc, yc, zc)):
            a[q] = src[q, order]
    return out


def write_re2(path, xc, yc, zc, bcs, version="#v002", big_endian=False, curves=(),
              groups=None, extra_bc_sections=()):
    """Write a 3-D .re2 file: header, byte-order test value, element records,
    curved sides, boundary sections (the first from bcs, then any extra)."""
    nel = xc.shape[0]
    wd = 4 if version == "#v001" else 8
    e = ">" if big_endian else "<"
    real = e + ("d" if wd == 8 else "f")
    integer = real if wd == 8 else e + "i"

    def w_int(v):
        return struct.pack(integer, float(v) if wd == 8 else int(v))

    def w_real(v):
        return struct.pack(real, v)

    out = bytearray()
    hdr = f"{version}{nel:9d}{3:3d}{nel:9d} hdr".ljust(80)
    out += hdr.encode()
    out += struct.pack(e + "f", 6.54321)
    for q in range(nel):
        out += w_int(0 if groups is None else groups[q])
        for arr in (xc, yc, zc):
            for c in range(8):
                out += w_real(arr[q, c])
    out += w_int(len(curves))
    for (el, side, vals, t) in curves:
        out += w_int(el) + w_int(side) + b"".join(w_real(v) for v in vals)
        out += t.encode().ljust(wd)
    for sec in (bcs,) + tuple(extra_bc_sections):
        out += w_int(len(sec))
        for (el, f, vals, t) in sec:
            out += w_int(el) + w_int(f) + b"".join(w_real(v) for v in vals)
            out += t.encode().ljust(wd)
    with open(path, "wb") as fh:
        fh.write(bytes(out))


def same_partition(a, b):
    """True when two id arrays group positions identically."""
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    _, ia = np.unique(a, return_inverse=True)
    _, ib = np.unique(b, return_inverse=True)
    # first-occurrence relabelling
    def canon(i):
        first = {}
        return np.array([first.setdefault(v, len(first)) for v in i])
    return np.array_equal(canon(ia), canon(ib))
