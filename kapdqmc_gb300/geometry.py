"""Lattice geometry of the two-sublattice lattices used by the sweep.

Host-side set-up, run once per model.  Indices follow the reference's
1-based convention (site ``i`` in ``1..Ns``; odd ``i`` = sublattice A,
even ``i`` = sublattice B of the same unit cell) so that bond lists and
fields exchanged with a Julia caller need no translation.

Reference: src/public/Geometry.jl (KAPDQMC).
"""
from __future__ import annotations

import numpy as np

LATTICES = ("SQUARE45", "SQUARE90", "HoneyComb120", "HoneyComb60")


def _mod1(x: int, n: int) -> int:
    """Julia's ``mod1``: result in ``1..n``."""
    return (x - 1) % n + 1


def xy_i(site, x: int, y: int) -> int:
    """(x, y) unit-cell coordinate -> index of its B (even) site.

    Reference: src/public/Geometry.jl:8-13 (the range check there can never
    fire; a real check is done here).
    """
    if not (1 <= x <= site[0] and 1 <= y <= site[1]):
        raise ValueError("Error : Out of Lattice Range!")
    return 2 * (x + (y - 1) * site[0])


def i_xy(site, i: int):
    """Site index -> unit-cell coordinate (x, y).  src/public/Geometry.jl:18-21."""
    j = -(-i // 2)
    return _mod1(j, site[0]), -(-j // site[0])


def nn2idx(lattice: str, site, idx: int):
    """Nearest neighbours of site ``idx`` (1-based), in the reference's order.

    Reference: src/public/Geometry.jl:74-134.
    """
    if len(site) == 1:
        return [_mod1(idx - 1, site[0]), _mod1(idx + 1, site[0])]
    x, y = i_xy(site, idx)
    L1, L2 = site[0], site[1]
    odd = idx % 2 == 1
    if lattice == "SQUARE90":
        if odd:
            return [idx + 1,
                    xy_i(site, _mod1(x - 1, L1), _mod1(y - 1, L2)),
                    xy_i(site, x, _mod1(y - 1, L2)),
                    xy_i(site, _mod1(x - 1, L1), y)]
        return [xy_i(site, _mod1(x + 1, L1), y) - 1,
                xy_i(site, x, _mod1(y + 1, L2)) - 1,
                idx - 1,
                xy_i(site, _mod1(x + 1, L1), _mod1(y + 1, L2)) - 1]
    if lattice == "SQUARE45":
        if odd:
            return [xy_i(site, _mod1(x - 1, L1), y),                      # left
                    idx + 1,                                              # right
                    xy_i(site, _mod1(x - 1, L1), _mod1(y + 1, L2)),       # up
                    xy_i(site, x, _mod1(y - 1, L2))]                      # down
        return [xy_i(site, x, _mod1(y + 1, L2)) - 1,                      # up
                xy_i(site, _mod1(x + 1, L1), _mod1(y - 1, L2)) - 1,       # down
                idx - 1,                                                  # left
                xy_i(site, _mod1(x + 1, L1), y) - 1]                      # right
    if lattice == "HoneyComb120":
        if odd:
            return [idx + 1,
                    xy_i(site, _mod1(x + 1, L1), y),
                    xy_i(site, x, _mod1(y - 1, L2))]
        return [idx - 1,
                xy_i(site, x, _mod1(y + 1, L2)) - 1,
                xy_i(site, _mod1(x - 1, L1), y) - 1]
    if lattice == "HoneyComb60":
        if odd:
            return [idx + 1,
                    xy_i(site, _mod1(x + 1, L1), _mod1(y - 1, L2)),
                    xy_i(site, x, _mod1(y - 1, L2))]
        return [idx - 1,
                xy_i(site, x, _mod1(y + 1, L2)) - 1,
                xy_i(site, _mod1(x - 1, L1), _mod1(y + 1, L2)) - 1]
    raise ValueError(f"Lattice: {lattice} is not allowed !")


def nnidx_F(lattice: str, site):
    """Bond list: ``(Ns/2) x z`` array of 1-based ``(A, B)`` pairs.

    Row ``i`` is the i-th A site (odd index ``2i-1``), column ``j`` its j-th
    neighbour as ordered by :func:`nn2idx`.  Each column is a perfect matching
    of the lattice.  Reference: src/public/Geometry.jl:24-66 (honeycomb
    branch).  The square lattices are accepted here as well (the reference
    only knows the unnamed "SQUARE", which its own ``nn2idx`` rejects); the
    same rule - every odd site with all its neighbours - is applied.
    """
    if lattice not in LATTICES:
        raise ValueError(f"Lattice: {lattice} is not allowed !")
    ns_ = 2 * int(np.prod(site))
    z = 3 if "HoneyComb" in lattice else 4
    out = np.zeros((ns_ // 2, z, 2), dtype=np.int64)
    for r, i in enumerate(range(1, ns_ + 1, 2)):
        nn = nn2idx(lattice, site, i)
        for j in range(z):
            out[r, j] = (i, nn[j])
    return out


def nnK_Matrix(lattice: str, site, t=(1.0, 1.0, 1.0), flux: float = 0.0):
    """Hopping matrix K (Ns x Ns), real unless a flux is threaded.

    Reference: src/public/Geometry.jl:178-207.
    """
    ns_ = int(np.prod(site)) * 2
    if flux == 0:
        K = np.zeros((ns_, ns_), dtype=np.float64)
        f1 = f2 = 1.0
    else:
        K = np.zeros((ns_, ns_), dtype=np.complex128)
        f1, f2 = np.exp(1j * flux / 4), np.exp(-1j * flux / 4)
    if "SQUARE" in lattice:
        for i in range(1, ns_ + 1):
            nn = nn2idx(lattice, site, i)
            K[i - 1, nn[0] - 1] = f1
            K[i - 1, nn[1] - 1] = f1
            K[i - 1, nn[2] - 1] = f2
            K[i - 1, nn[3] - 1] = f2
    elif "HoneyComb" in lattice:
        for i in range(1, ns_ + 1):
            nn = nn2idx(lattice, site, i)
            for j, n in enumerate(nn):
                K[i - 1, n - 1] = t[j]
    else:
        raise ValueError(f"Lattice: {lattice} is not allowed !")
    if np.linalg.norm(K - K.conj().T) >= 1e-8:
        raise AssertionError("K is not Hermitian!")
    return K


def area_index(lattice: str, site, area):
    """1-based site indices of a rectangular entanglement region.

    ``area = ((x0, y0), (x1, y1))`` in unit-cell coordinates.
    Reference: src/public/Geometry.jl:209-307 (SQUARE45, SQUARE90 and the
    rectangular honeycomb branch).
    """
    (a0, a1) = area
    if len(site) == 1:
        return list(range(a0[0], a1[0] + 1))
    if lattice == "SQUARE45":
        Nx, Ny = a1[0] - a0[0] + 1, a1[1] - a0[1] + 1
        if Nx > 2 * site[0] or Ny > site[1]:
            raise ValueError("Error : Out of Lattice Range!")
        start = xy_i(site, a0[0], a0[1]) - 1
        typeS = typ = "A"
        index = [start]
        for yy in range(1, Ny + 1):
            point = start
            for _ in range(Nx - 1):
                if typ == "A":
                    point = nn2idx(lattice, site, point)[1]
                    typ = "B"
                else:
                    point = nn2idx(lattice, site, point)[3]
                    typ = "A"
                index.append(point)
            if yy != Ny:
                if typeS == "A":
                    start = nn2idx(lattice, site, start)[2]
                    typeS = typ = "B"
                else:
                    start = nn2idx(lattice, site, start)[0]
                    typeS = typ = "A"
                index.append(start)
        return index
    if lattice == "SQUARE90" or "HoneyComb" in lattice:
        index = []
        for lx in range(a0[0], a1[0] + 1):
            for ly in range(a0[1], a1[1] + 1):
                b = xy_i(site, lx, ly) - 1
                index += [b, b + 1]
        return index
    raise ValueError(f"Lattice: {lattice} is not allowed !")
