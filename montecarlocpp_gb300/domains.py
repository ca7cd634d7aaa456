"""Domain descriptions: assemblies of Parallelepiped subdomains.

A montecarlocpp Domain is a set of ``Parallelepiped<Bac, Lef, Bot, Fro, Rig,
Top>`` subdomains (montecarlo/subdomain.h:128-198) joined by ``makePair``
calls (Inter pairs montecarlo/boundary.cpp:361-369, Peri pairs
montecarlo/boundary.cpp:524-550). This module keeps exactly those primitive
constructor arguments -- origin, edge matrix, divisions, volumetric
temperature gradient, the kind and temperature of each face, and the pair
list -- and nothing derived from them; the library derives normals, plane
offsets, rotations, emitter weights and field strides itself.

Faces are numbered as the reference's ``bdry<I>()``: 0 Bac (origin, edges
col1 x col2), 1 Lef, 2 Bot, 3 Fro (origin + col0), 4 Rig, 5 Top.

FilmDomain and BulkDomain restate montecarlo/domain.cpp:137-199. The
cross-plane film and the periodic pore cell are assembled only from the
reference's public building blocks (Parallelepiped, IsotBoundary,
SpecBoundary, DiffBoundary, InterBoundary, PeriBoundary, makePair).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SPEC, DIFF, ISOT, PERI, INTER = 0, 1, 2, 3, 4
KIND_NAMES = {SPEC: "Spec", DIFF: "Diff", ISOT: "Isot", PERI: "Peri", INTER: "Inter"}
BAC, LEF, BOT, FRO, RIG, TOP = range(6)

__all__ = [
    "SPEC", "DIFF", "ISOT", "PERI", "INTER", "BAC", "LEF", "BOT", "FRO", "RIG", "TOP",
    "Parallelepiped", "Pair", "Domain", "FilmDomain", "BulkDomain",
    "CrossPlaneFilmDomain", "PoreCellDomain",
]


@dataclass
class Parallelepiped:
    o: np.ndarray
    M: np.ndarray  # 3x3, columns are the edge vectors
    div: np.ndarray  # 3 longs
    gradT: np.ndarray
    kinds: tuple  # 6 face kinds
    T: tuple = (0.0,) * 6

    def shape(self):
        d = np.asarray(self.div)
        if (d < 0).any():
            return np.zeros(3, dtype=np.int64)
        return np.maximum(d, 1).astype(np.int64)

    def vol(self) -> float:
        return float(np.linalg.det(self.M))


@dataclass
class Pair:
    kind: int  # PERI or INTER
    s1: int
    f1: int
    s2: int
    f2: int
    transl: np.ndarray = field(default_factory=lambda: np.zeros(3))
    rot: np.ndarray = field(default_factory=lambda: np.eye(3))


class Domain:
    """A domain as a list of parallelepipeds and a list of pairs."""

    name = "Domain"

    def __init__(self, ppeds, pairs):
        self.ppeds = list(ppeds)
        self.pairs = list(pairs)
        self._check()

    def _check(self):
        for p in self.ppeds:
            if not (p.vol() >= np.finfo(float).tiny):
                raise ValueError("Volume too small, check vector order")
            for k, T in zip(p.kinds, p.T):
                if k in (SPEC, DIFF, INTER) and T != 0.0:
                    raise ValueError("Cannot specify temperature")
        used = set()
        for q in self.pairs:
            for s, f in ((q.s1, q.f1), (q.s2, q.f2)):
                if self.ppeds[s].kinds[f] != q.kind:
                    raise ValueError("pair kind does not match face kind")
                if q.kind == PERI:
                    if (s, f) in used:
                        raise ValueError("Boundary already paired")
                    used.add((s, f))
        for i, p in enumerate(self.ppeds):
            for f, k in enumerate(p.kinds):
                if k in (PERI, INTER):
                    if not any((q.s1, q.f1) == (i, f) or (q.s2, q.f2) == (i, f) for q in self.pairs):
                        raise ValueError("Domain setup not complete: unpaired face")

    def cols(self) -> int:
        return int(sum(int(np.prod(p.shape())) for p in self.ppeds))

    def cell_volumes(self) -> np.ndarray:
        out = []
        for p in self.ppeds:
            n = int(np.prod(p.shape()))
            if n:
                out.extend([p.vol() / n] * n)
        return np.array(out)

    def max_dim(self) -> float:
        return max(float(np.linalg.norm(p.M[:, c])) for p in self.ppeds for c in range(3))


def _pped(o, dims, div, gradT, kinds, T=(0.0,) * 6):
    return Parallelepiped(np.asarray(o, dtype=np.float64), np.diag(np.asarray(dims, dtype=np.float64)),
                          np.asarray(div, dtype=np.int64), np.asarray(gradT, dtype=np.float64),
                          tuple(kinds), tuple(float(t) for t in T))


class FilmDomain(Domain):
    """In-plane film: PeriP along x, Diff along y (the thickness), Spec
    along z (montecarlo/domain.cpp:188-199, type montecarlo/domain.h:119).
    The CLI uses dim = (Lx, thickness, Lx), div = (0, ncell, 0) and
    dT = 1e6 * Lx, i.e. a 1 K/um gradient (montecarlo/main.cpp:309-318)."""

    name = "FilmDomain"

    def __init__(self, dim, div, dT):
        dim = np.asarray(dim, dtype=np.float64)
        self.dim, self.div, self.dT = dim, np.asarray(div, dtype=np.int64), float(dT)
        p = _pped((0, 0, 0), dim, div, (-dT / dim[0], 0, 0), (PERI, DIFF, SPEC, PERI, DIFF, SPEC))
        q = Pair(PERI, 0, BAC, 0, FRO, np.array([dim[0], 0.0, 0.0]))
        super().__init__([p], [q])

    @classmethod
    def from_cli(cls, Lx, thickness, ncell):
        return cls((Lx, thickness, Lx), (0, ncell, 0), 1e6 * Lx)


class BulkDomain(Domain):
    """Bulk: PeriP along x, Spec along y and z (montecarlo/domain.cpp:137-148);
    the CLI uses a cube of side dim0, div = (ndiv, 0, 0), dT = 1e6 * dim0."""

    name = "BulkDomain"

    def __init__(self, dim, div, dT):
        dim = np.asarray(dim, dtype=np.float64)
        self.dim, self.div, self.dT = dim, np.asarray(div, dtype=np.int64), float(dT)
        p = _pped((0, 0, 0), dim, div, (-dT / dim[0], 0, 0), (PERI, SPEC, SPEC, PERI, SPEC, SPEC))
        q = Pair(PERI, 0, BAC, 0, FRO, np.array([dim[0], 0.0, 0.0]))
        super().__init__([p], [q])

    @classmethod
    def from_cli(cls, dim0, ndiv):
        return cls((dim0, dim0, dim0), (ndiv, 0, 0), 1e6 * dim0)


class CrossPlaneFilmDomain(Domain):
    """Cross-plane film between two isothermal walls:
    ``Parallelepiped<IsotBoundary<Parallelogram>, Spec, Spec>`` with face
    temperatures (T_hot, 0, 0, T_cold, 0, 0) relative to the linearisation
    temperature; no volumetric source. Walls emit with weight area*|T| and
    absorb (montecarlo/boundary.cpp:413-460)."""

    name = "CrossPlaneFilmDomain"

    def __init__(self, L, width, ncell, T_hot=1.0, T_cold=-1.0):
        self.L, self.width, self.ncell = float(L), float(width), int(ncell)
        p = _pped((0, 0, 0), (L, width, width), (ncell, 0, 0), (0, 0, 0),
                  (ISOT, SPEC, SPEC, ISOT, SPEC, SPEC), (T_hot, 0, 0, T_cold, 0, 0))
        super().__init__([p], [])


class PoreCellDomain(Domain):
    """Periodic cubic cell of side `side` with a centred cubic void of side
    `void`: 26 Parallelepipeds (a 3x3x3 block grid minus the centre) joined
    by InterBoundary pairs, PeriP pairs on the outer faces along x, y and z,
    DiffBoundary on the six pore walls, and a volumetric gradient
    (-dT / side, 0, 0) in every block. `divs` gives the cell divisions of
    the three block widths along each axis (default 12, 26, 12: a 50^3 grid
    of near-10-nm cells for a 500 nm cell with a 250 nm pore)."""

    name = "PoreCellDomain"

    def __init__(self, side, void, divs=(12, 26, 12), dT=None):
        side, void = float(side), float(void)
        if not (0 < void < side):
            raise ValueError("void must be inside the cell")
        dT = 1e6 * side if dT is None else float(dT)
        self.side, self.void, self.divs, self.dT = side, void, tuple(divs), dT
        w = [(side - void) / 2, void, (side - void) / 2]
        x0 = [0.0, w[0], w[0] + w[1]]
        index = {}
        ppeds = []
        for k in range(3):
            for j in range(3):
                for i in range(3):
                    if (i, j, k) == (1, 1, 1):
                        continue
                    index[(i, j, k)] = len(ppeds)
                    ppeds.append(None)
        pairs = []

        def nb(i, j, k):
            return index.get((i, j, k))

        for (i, j, k), s in index.items():
            ijk = (i, j, k)
            kinds = [None] * 6
            for axis in range(3):
                lo, hi = axis, axis + 3
                for face, step in ((lo, -1), (hi, +1)):
                    n = list(ijk)
                    n[axis] += step
                    if n[axis] < 0 or n[axis] > 2:
                        kinds[face] = PERI
                    elif tuple(n) == (1, 1, 1):
                        kinds[face] = DIFF
                    else:
                        kinds[face] = INTER
            ppeds[s] = _pped((x0[i], x0[j], x0[k]), (w[i], w[j], w[k]),
                             (divs[i], divs[j], divs[k]), (-dT / side, 0, 0), kinds)
        for (i, j, k), s in index.items():
            ijk = (i, j, k)
            for axis in range(3):
                n = list(ijk)
                n[axis] += 1
                if n[axis] <= 2 and tuple(n) != (1, 1, 1):
                    pairs.append(Pair(INTER, s, axis + 3, nb(*n), axis))
                if ijk[axis] == 0:
                    m = list(ijk)
                    m[axis] = 2
                    t = np.zeros(3)
                    t[axis] = side
                    pairs.append(Pair(PERI, s, axis, nb(*m), axis + 3, t))
        super().__init__(ppeds, pairs)
