"""Domain descriptions: assemblies of subdomains.

A montecarlocpp Domain is a set of subdomains -- ``Parallelepiped``,
``TriangularPrism``, ``Tetrahedron``, ``Prism<N>`` and ``Pyramid<N>``
(montecarlo/subdomain.h:128-640) -- joined by ``makePair`` calls (Inter
pairs montecarlo/boundary.cpp:361-369, Peri pairs
montecarlo/boundary.cpp:524-550). This module keeps exactly those primitive
constructor arguments -- origin, edge matrix, divisions, volumetric
temperature gradient, the kind and temperature of each face, and the pair
list -- and nothing derived from them; the library derives normals, plane
offsets, rotations, emitter weights and field strides itself.

Faces are numbered as the reference's ``bdry<I>()``. Parallelepiped: 0 Bac
(origin, edges col1 x col2), 1 Lef, 2 Bot, 3 Fro (origin + col0), 4 Rig, 5
Top. TriangularPrism: Bac, Lef, Bot, Dia, Top. Tetrahedron: Bac, Lef, Bot,
Dia. Prism<N>: Bot, Top, then the N sides. Pyramid<N>: Bot, then the N
sides.

FilmDomain, BulkDomain, PyrDomain, HexDomain, JctDomain, TeeDomain and
TubeDomain restate montecarlo/domain.cpp:137-570. The cross-plane film and
the periodic pore cell are assembled only from the reference's public
building blocks (Parallelepiped, IsotBoundary, SpecBoundary, DiffBoundary,
InterBoundary, PeriBoundary, makePair).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SPEC, DIFF, ISOT, PERI, INTER = 0, 1, 2, 3, 4
KIND_NAMES = {SPEC: "Spec", DIFF: "Diff", ISOT: "Isot", PERI: "Peri", INTER: "Inter"}
BAC, LEF, BOT, FRO, RIG, TOP = range(6)
PARALLELEPIPED, TRIANGULAR_PRISM, TETRAHEDRON, PRISM, PYRAMID = range(5)

__all__ = [
    "SPEC", "DIFF", "ISOT", "PERI", "INTER", "BAC", "LEF", "BOT", "FRO", "RIG", "TOP",
    "PARALLELEPIPED", "TRIANGULAR_PRISM", "TETRAHEDRON", "PRISM", "PYRAMID",
    "Parallelepiped", "TriangularPrism", "Tetrahedron", "Prism", "Pyramid", "Pair", "Domain",
    "FilmDomain", "BulkDomain", "CrossPlaneFilmDomain", "PoreCellDomain", "PyrDomain", "HexDomain",
    "JctDomain", "TeeDomain", "TubeDomain", "OctetDomain",
]


@dataclass
class Parallelepiped:
    o: np.ndarray
    M: np.ndarray  # 3x3, columns are the edge vectors
    div: np.ndarray  # 3 longs
    gradT: np.ndarray
    kinds: tuple  # 6 face kinds
    T: tuple = (0.0,) * 6

    shape_kind = PARALLELEPIPED

    def shape(self):
        d = np.asarray(self.div)
        if (d < 0).any():
            return np.zeros(3, dtype=np.int64)
        return np.maximum(d, 1).astype(np.int64)

    def vol(self) -> float:
        return float(np.linalg.det(self.M))

    def columns(self) -> np.ndarray:
        return np.asarray(self.M, dtype=np.float64)

    def divisions(self) -> np.ndarray:
        return np.asarray(self.div, dtype=np.int64)


@dataclass
class TriangularPrism(Parallelepiped):
    """TriangularPrism<Bac, Lef, Bot, Dia, Top>(o, mat, div, gradT, T)
    (montecarlo/subdomain.h:207-279): the half of the parallelepiped
    (o, mat) below the diagonal plane through o + col0 and o + col1; the
    cells are those of the parallelepiped grid."""

    T: tuple = (0.0,) * 5
    shape_kind = TRIANGULAR_PRISM

    def vol(self) -> float:
        return float(np.linalg.det(self.M)) / 2.0


@dataclass
class Tetrahedron(Parallelepiped):
    """Tetrahedron<Bac, Lef, Bot, Dia>(o, mat, div, gradT, T)
    (montecarlo/subdomain.h:286-358): vertices o, o + col0, o + col1,
    o + col2."""

    T: tuple = (0.0,) * 4
    shape_kind = TETRAHEDRON

    def vol(self) -> float:
        return float(np.linalg.det(self.M)) / 6.0


@dataclass
class Prism:
    """Prism<Bot, Top, Sid...>(o, mat, div, gradT, T)
    (montecarlo/subdomain.h:365-503): mat is 3 x N, column 0 the axis and
    columns 1 .. N-1 the base vertices after o; div < 0 gives no field,
    otherwise one column for the whole prism."""

    o: np.ndarray
    mat: np.ndarray
    div: int
    gradT: np.ndarray
    kinds: tuple  # N + 2 face kinds: Bot, Top, sides
    T: tuple = None

    shape_kind = PRISM
    _per = 2.0

    def __post_init__(self):
        if self.T is None:
            self.T = (0.0,) * len(self.kinds)

    def columns(self) -> np.ndarray:
        return np.asarray(self.mat, dtype=np.float64)

    def divisions(self) -> np.ndarray:
        return np.array([self.div, 0, 0], dtype=np.int64)

    def shape(self):
        return np.zeros(3, dtype=np.int64) if self.div < 0 else np.ones(3, dtype=np.int64)

    def vol(self) -> float:
        # PrismImpl::volume / PyramidImpl::volume (montecarlo/subdomain.cpp:
        # 384-392,416-424), summed as the reference sums them
        m = self.columns()
        n = m.shape[1]
        return float(sum(np.dot(np.cross(m[:, i], m[:, i + 1]), m[:, 0]) for i in range(n - 2)) / self._per)


@dataclass
class Pyramid(Prism):
    """Pyramid<Bot, Sid...>(o, mat, div, gradT, T)
    (montecarlo/subdomain.h:505-640): column 0 the apex, columns 1 .. N-1
    the base vertices after o."""

    shape_kind = PYRAMID
    _per = 6.0


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
        """Cell volumes of Parallelepiped-only domains (other shapes: the
        library's mc_domain_cell_volumes)."""
        out = []
        for p in self.ppeds:
            if p.shape_kind != PARALLELEPIPED:
                raise ValueError("cell volumes of this shape come from the library")
            n = int(np.prod(p.shape()))
            if n:
                out.extend([p.vol() / n] * n)
        return np.array(out)

    def max_dim(self) -> float:
        return max(float(np.linalg.norm(p.columns()[:, c])) for p in self.ppeds
                   for c in range(p.columns().shape[1]))

    def parallelepipeds_only(self) -> bool:
        return all(p.shape_kind == PARALLELEPIPED for p in self.ppeds)


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


class PyrDomain(Domain):
    """Square pyramid with specular walls and a volumetric gradient along
    its axis: ``Pyramid<Spec, Spec x 4>`` (montecarlo/domain.cpp:299-314,
    type montecarlo/domain.h:162-165); the CLI uses dim = (height, base,
    base) and dT = 1e6 * height (montecarlo/main.cpp:330-337)."""

    name = "PyrDomain"

    def __init__(self, dim, dT):
        dim = np.asarray(dim, dtype=np.float64)
        self.dim, self.dT = dim, float(dT)
        mat = np.array([[dim[0], 0.5 * dim[1], 0.5 * dim[2]],
                        [0.0, dim[1], 0.0],
                        [0.0, dim[1], dim[2]],
                        [0.0, 0.0, dim[2]]]).T
        p = Pyramid(np.zeros(3), mat, 0, np.array([-dT / dim[0], 0.0, 0.0]), (SPEC,) * 5)
        super().__init__([p], [])

    @classmethod
    def from_cli(cls, height, base):
        return cls((height, base, base), 1e6 * height)


class HexDomain(Domain):
    """Hexagonal rod, periodic along its axis with specular sides:
    ``Prism<PeriP<Polygon<6>>, PeriP<Polygon<6>>, Spec x 6>``
    (montecarlo/domain.cpp:238-256, type montecarlo/domain.h:139-142); the
    CLI uses dim = (length, d, d, d) and dT = 1e6 * length
    (montecarlo/main.cpp:320-328). Eight faces: the kernels keep the last
    two in a continuation slot."""

    name = "HexDomain"

    def __init__(self, dim, dT):
        dim = np.asarray(dim, dtype=np.float64)
        self.dim, self.dT = dim, float(dT)
        mat = np.array([[dim[0], 0.0, 0.0],
                        [0.0, dim[1], -dim[3]],
                        [0.0, 2.0 * dim[1], 0.0],
                        [0.0, 2.0 * dim[1], dim[2]],
                        [0.0, dim[1], dim[2] + dim[3]],
                        [0.0, 0.0, dim[2]]]).T
        p = Prism(np.zeros(3), mat, 0, np.array([-dT / dim[0], 0.0, 0.0]), (PERI, PERI) + (SPEC,) * 6)
        q = Pair(PERI, 0, 0, 0, 1, np.array([dim[0], 0.0, 0.0]))
        super().__init__([p], [q])

    @classmethod
    def from_cli(cls, length, d):
        return cls((length, d, d, d), 1e6 * length)


class JctDomain(Domain):
    """L-junction of three blocks (montecarlo/domain.cpp:353-383, type
    montecarlo/domain.h:184-190): block 0's Rig face pairs with two Inter
    faces, so a phonon crossing it goes to the first block that contains
    it (montecarlo/boundary.cpp:349-359); the kernels test the candidates
    in that order."""

    name = "JctDomain"

    def __init__(self, dim, div, dT):
        d = np.asarray(dim, dtype=np.float64)
        v = np.asarray(div, dtype=np.int64)
        self.dim, self.div, self.dT = d, v, float(dT)
        g = (-dT / (2.0 * d[0]), 0.0, 0.0)
        p0 = _pped((0, 0, 0), (2 * d[0], d[1], d[3]), (2 * v[0], v[1], v[3]), g,
                   (PERI, SPEC, DIFF, PERI, INTER, DIFF))
        p1 = _pped((0, d[1], 0), (d[0], d[2], d[3]), (v[0], v[2], v[3]), g, (PERI, INTER, DIFF, INTER, SPEC, DIFF))
        p2 = _pped((d[0], d[1], 0), (d[0], d[2], d[3]), (v[0], v[2], v[3]), g,
                   (INTER, INTER, DIFF, PERI, SPEC, DIFF))
        t = np.array([2.0 * d[0], 0.0, 0.0])
        pairs = [Pair(INTER, 0, RIG, 1, LEF), Pair(INTER, 0, RIG, 2, LEF), Pair(INTER, 1, FRO, 2, BAC),
                 Pair(PERI, 0, BAC, 0, FRO, t), Pair(PERI, 1, BAC, 2, FRO, t)]
        super().__init__([p0, p1, p2], pairs)

    @classmethod
    def from_cli(cls, d0, d3):
        return cls((d0, d0, d0, d3), (0, 0, 0, 0), 2e6 * d0)


class TeeDomain(Domain):
    """T-junction of four blocks (montecarlo/domain.cpp:430-462, type
    montecarlo/domain.h:213-220); the CLI uses dim = (d, d, d, d, w),
    div = (n, n, n, n, 0) and dT = 3e6 * d (montecarlo/main.cpp:350-362)."""

    name = "TeeDomain"

    def __init__(self, dim, div, dT):
        d = np.asarray(dim, dtype=np.float64)
        v = np.asarray(div, dtype=np.int64)
        self.dim, self.div, self.dT = d, v, float(dT)
        g = (-dT / (2.0 * d[0] + d[1]), 0.0, 0.0)
        p0 = _pped((0, 0, 0), (d[0], d[2], d[4]), (v[0], v[2], v[4]), g, (PERI, DIFF, SPEC, INTER, DIFF, SPEC))
        p1 = _pped((d[0], 0, 0), (d[1], d[2], d[4]), (v[1], v[2], v[4]), g, (INTER, SPEC, SPEC, INTER, INTER, SPEC))
        p2 = _pped((d[0], d[2], 0), (d[1], d[3], d[4]), (v[1], v[3], v[4]), g, (DIFF, INTER, SPEC, DIFF, SPEC, SPEC))
        p3 = _pped((d[0] + d[1], 0, 0), (d[0], d[2], d[4]), (v[0], v[2], v[4]), g,
                   (INTER, DIFF, SPEC, PERI, DIFF, SPEC))
        pairs = [Pair(INTER, 0, FRO, 1, BAC), Pair(INTER, 1, RIG, 2, LEF), Pair(INTER, 1, FRO, 3, BAC),
                 Pair(PERI, 0, BAC, 3, FRO, np.array([2.0 * d[0] + d[1], 0.0, 0.0]))]
        super().__init__([p0, p1, p2, p3], pairs)

    @classmethod
    def from_cli(cls, d0, w, n):
        return cls((d0, d0, d0, d0, w), (n, n, n, n, 0), 3e6 * d0)


class TubeDomain(Domain):
    """Square tube of three blocks around an open corner, periodic along x
    (montecarlo/domain.cpp:510-540, type montecarlo/domain.h:262-269); the
    CLI uses dim = (L, a, a, t), div = (0, n, n, m) and dT = 1e6 * L
    (montecarlo/main.cpp:364-374)."""

    name = "TubeDomain"

    def __init__(self, dim, div, dT):
        d = np.asarray(dim, dtype=np.float64)
        v = np.asarray(div, dtype=np.int64)
        self.dim, self.div, self.dT = d, v, float(dT)
        g = (-dT / d[0], 0.0, 0.0)
        p0 = _pped((0, d[1], 0), (d[0], d[3], d[2]), (v[0], v[3], v[2]), g, (PERI, DIFF, SPEC, PERI, DIFF, INTER))
        p1 = _pped((0, d[1], d[2]), (d[0], d[3], d[3]), (v[0], v[3], v[3]), g, (PERI, INTER, INTER, PERI, DIFF, DIFF))
        p2 = _pped((0, 0, d[2]), (d[0], d[1], d[3]), (v[0], v[1], v[3]), g, (PERI, SPEC, DIFF, PERI, INTER, DIFF))
        t = np.array([d[0], 0.0, 0.0])
        pairs = [Pair(INTER, 1, LEF, 2, RIG), Pair(INTER, 1, BOT, 0, TOP),
                 Pair(PERI, 0, BAC, 0, FRO, t), Pair(PERI, 1, BAC, 1, FRO, t), Pair(PERI, 2, BAC, 2, FRO, t)]
        super().__init__([p0, p1, p2], pairs)

    @classmethod
    def from_cli(cls, L, a, t, n, m):
        return cls((L, a, a, t), (0, n, n, m), 1e6 * L)


class OctetDomain(Domain):
    """One cell of an octet-truss lattice (montecarlo/domain.cpp:591-1238,
    types montecarlo/domain.h:298-344): 42 subdomains -- Prism<4> slabs
    and nodes, TriangularPrisms, Pyramids and Parallelepipeds -- joined by
    Inter pairs (ten faces paired with two others), with five Peri pairs
    mapped by the reflection diag(-1, 1, 1) and the translation
    (s/2, 0, -s/2). The ten vertical struts (16-25) carry the cells and the
    gradient. dim = (s, d1, d2, t): a = pi/5 (d1 + d2) - (4 - pi)/5 t and
    b = a/4; div = (div0 .. div3) as the reference's CLI `octet` takes them
    (montecarlo/main.cpp:376-386)."""

    name = "OctetDomain"
    # face kinds per subdomain in bdry<I>() order (Prism: Bot, Top, sides;
    # Pyramid: Bot, sides; TriangularPrism: Bac, Lef, Bot, Dia, Top)
    _I, _D, _S, _P = INTER, DIFF, SPEC, PERI
    KINDS = [
        (_I, _P, _I, _D, _S, _D), (_D, _I, _I, _D, _S, _I), (_D, _D, _I, _I, _S, _S), (_I, _P, _D, _I, _I, _D),
        (_I, _I, _D, _I, _I, _I), (_I, _S, _D, _D, _I, _I), (_S, _I, _P, _D, _I, _D), (_I, _D, _P, _D, _I, _I),
        (_D, _D, _P, _I, _I, _I), (_D, _D, _I, _I, _I, _I), (_I, _D, _I, _I, _D, _I), (_S, _I, _D, _I, _D, _I),
        (_D, _I, _I, _S, _I), (_I, _D, _I, _S, _I), (_I, _I, _D, _S, _I), (_D, _D, _I, _I, _S, _S),
        (_D, _S, _I, _D, _I, _I), (_I, _I, _I, _D, _D, _I), (_I, _D, _I, _I, _D, _I), (_D, _I, _I, _I, _D, _I),
        (_D, _S, _I, _D, _I, _I), (_D, _S, _I, _D, _I, _I), (_D, _I, _I, _I, _D, _I), (_I, _D, _I, _I, _D, _I),
        (_I, _I, _I, _D, _D, _I), (_D, _S, _I, _D, _I, _I), (_D, _D, _I, _I, _S, _S), (_I, _I, _D, _S, _I),
        (_I, _D, _I, _S, _I), (_D, _I, _I, _S, _I), (_S, _I, _D, _I, _D, _I), (_I, _D, _I, _I, _D, _I),
        (_D, _D, _I, _I, _I, _I), (_D, _D, _P, _I, _I, _I), (_I, _D, _P, _D, _I, _I), (_S, _I, _P, _D, _I, _D),
        (_I, _S, _D, _D, _I, _I), (_I, _I, _D, _I, _I, _I), (_I, _P, _D, _I, _I, _D), (_D, _D, _I, _I, _S, _S),
        (_D, _I, _I, _D, _S, _I), (_I, _P, _I, _D, _S, _D),
    ]
    INTER_PAIRS = [
        (0, 0, 1, 1), (1, 5, 2, 3), (0, 2, 3, 4), (1, 2, 4, 4), (2, 2, 5, 5), (3, 0, 4, 1), (4, 5, 5, 4),
        (3, 3, 8, 5), (4, 3, 8, 5), (4, 0, 9, 2), (5, 0, 9, 2), (5, 0, 12, 4),
        (6, 1, 7, 0), (7, 5, 8, 3), (9, 4, 10, 2), (10, 0, 11, 1), (9, 5, 12, 1), (9, 5, 13, 0), (10, 5, 14, 1),
        (11, 5, 15, 2), (12, 2, 13, 2), (13, 4, 14, 4), (14, 0, 15, 3),
        (6, 4, 16, 5), (7, 4, 17, 5), (8, 4, 18, 5), (9, 3, 18, 5), (10, 3, 19, 5), (11, 3, 20, 5),
        (16, 4, 17, 1), (17, 0, 18, 3), (18, 0, 19, 3), (19, 1, 20, 4),
        (16, 2, 21, 2), (17, 2, 22, 2), (18, 2, 23, 2), (19, 2, 24, 2), (20, 2, 25, 2),
        (21, 4, 22, 1), (22, 3, 23, 0), (23, 3, 24, 0), (24, 1, 25, 4),
        (21, 5, 30, 3), (22, 5, 31, 3), (23, 5, 32, 3), (23, 5, 33, 4), (24, 5, 34, 4), (25, 5, 35, 4),
        (26, 3, 27, 0), (27, 4, 28, 4), (28, 2, 29, 2), (26, 2, 30, 5), (27, 1, 31, 5), (28, 0, 32, 5),
        (29, 1, 32, 5), (30, 1, 31, 0), (31, 2, 32, 4), (33, 3, 34, 5), (34, 0, 35, 1),
        (29, 4, 36, 0), (32, 2, 36, 0), (32, 2, 37, 0), (33, 5, 37, 3), (33, 5, 38, 3),
        (36, 4, 37, 5), (37, 1, 38, 0), (36, 5, 39, 2), (37, 4, 40, 2), (38, 4, 41, 2), (39, 3, 40, 5),
        (40, 1, 41, 0),
    ]
    PERI_PAIRS = [(0, 1, 41, 1), (3, 1, 38, 1), (6, 2, 35, 2), (7, 2, 34, 2), (8, 2, 33, 2)]
    AVERAGED = range(16, 26)

    def __init__(self, dim, div, dT):
        d = np.asarray(dim, dtype=np.float64)
        v = np.asarray(div, dtype=np.int64)
        self.dim, self.div, self.dT = d, v, float(dT)
        r = np.sqrt(2.0)
        s = d[0]
        a = np.pi / 5.0 * (d[1] + d[2]) - (4.0 - np.pi) / 5.0 * d[3]
        b = a / 4.0
        t = d[3]
        if not (b > t and a > (r + 1) * (b + t) and s / 2 > a + (r + 1) * (b + t) + t):
            raise ValueError("Invalid dimensions")
        self.a, self.b, self.t = a, b, t
        den = s - 2 * a - 2 * (r + 1) * b - 2 * (2 + r) * t
        g = np.array([dT / den, 0.0, -dT / den])
        z = np.zeros(3)
        h = 0.5
        q1, q2 = (r + 1) * h, (2 + r) * h  # (sqrt2 + 1) / 2, (2 + sqrt2) / 2
        P = lambda o, *cols: ("prism", o, cols)
        Y = lambda o, *cols: ("pyr", o, cols)
        T3 = lambda o, *cols: ("tri", o, cols)
        B3 = lambda o, cols, dv=None: ("box", o, cols, dv)
        # slab ends shared by sdom 00/01 and 40/41, 02 and 39, nodes
        e0 = ((r * t, 0, 0), (s / 4 - (2 + r) * h * b - (2 - r) * h * t, s / 4 - (2 + r) * h * (b + t), 0),
              (s / 4 - (2 + r) * h * b - t, s / 4 - (2 + r) * h * b - t, 0))
        e3 = (((r + 1) * t, 0, 0), ((r + 1) * t, t, 0), (t, t, 0))
        e6 = ((r * t, 0, 0), (q1 * b + (r + 1) * t, 0, -q1 * b - t), (q1 * b + q2 * t, 0, -q1 * b - q2 * t))
        e10 = (((r - 1) * h * b + t / r, 0, -(r - 1) * h * b - t / r), ((r - 1) * h * b, 0, -(r - 1) * h * b - r * t),
               (0, 0, -r * t))
        up = (-s / 4 + a / 2 + q1 * b + q2 * t, 0, s / 4 - a / 2 - q1 * b - q2 * t)  # strut axis, top
        dn = (s / 4 - a / 2 - q1 * b - q2 * t, 0, -s / 4 + a / 2 + q1 * b + q2 * t)  # strut axis, bottom
        e30 = ((-(r - 1) * h * b - t / r, 0, (r - 1) * h * b + t / r), (-(r - 1) * h * b, 0, (r - 1) * h * b + r * t),
               (0, 0, r * t))
        e34 = ((-r * t, 0, 0), (-q1 * b - (r + 1) * t, 0, q1 * b + t), (-q1 * b - q2 * t, 0, q1 * b + q2 * t))
        e37 = ((-(r + 1) * t, 0, 0), (-(r + 1) * t, t, 0), (-t, t, 0))
        e40 = ((-r * t, 0, 0), (-s / 4 + (2 + r) * h * b + (2 - r) * h * t, s / 4 - (2 + r) * h * (b + t), 0),
               (-s / 4 + (2 + r) * h * b + t, s / 4 - (2 + r) * h * b - t, 0))
        ts = t / r
        dv = lambda i, j, k: (v[i], v[j], v[k])
        spec = [
            P(((r + 1) * b + t, b + t, -a), (0, 0, a), *e0),                                       # 00
            P(((r + 1) * b + t, b + t, -a - t), (0, 0, t), *e0),                                   # 01
            P((b + t, b + t, -a - t), (0, 0, t), (r * b, 0, 0),
              (s / 4 - (2 - r) * h * b - t, s / 4 - (2 + r) * h * b - t, 0), (s / 4 - b - t, s / 4 - b - t, 0)),  # 02
            P(((r + 1) * b, b, -a), (0, 0, a), *e3),                                               # 03
            P(((r + 1) * b, b, -a - t), (0, 0, t), *e3),                                           # 04
            B3((b, b, -a - t), ((0, 0, t), (r * b, 0, 0), (t, t, 0))),                            # 05
            P((a, 0, 0), (0, b, 0), *e6),                                                          # 06
            P((a, b, 0), (0, t, 0), *e6),                                                          # 07
            P(((r + 1) * (b + t), b, 0), (0, t, 0), (a - (r + 1) * (b + t), 0, 0),
              (a - q1 * b - t / r, 0, -q1 * b - q2 * t), (0, 0, -a - t)),                          # 08
            P((b + t, b, -a - t), (0, t, 0), (r * (b + t), 0, 0),
              ((r - 1) * h * b + t / r, 0, -q1 * b - t / r), (0, 0, -b)),                          # 09
            P((b + t, b, -a - b - t), (0, t, 0), *e10),                                            # 10
            P((b + t, 0, -a - b - t), (0, b, 0), *e10),                                            # 11
            T3((b + t, b, -a - b), (0, t, 0), (-t, 0, 0), (0, 0, b - t)),                         # 12
            Y((b + t, b, -a - b - t), (-t, 0, t), (0, 0, t), (0, t, t), (0, t, 0)),               # 13
            T3((b + t, b, -a - b - (r + 1) * t), (0, t, 0), (-t, 0, t), (0, 0, r * t)),           # 14
            P((b + t, 0, -a - b - (r + 1) * t), (0, 0, r * t), (0, b, 0), (-t, b, t), (-b - t, 0, b + t)),  # 15
            B3((s / 4 + a / 2, 0, -s / 4 + a / 2), ((ts, 0, ts), (0, b, 0), up), dv(3, 2, 0)),    # 16
            B3((s / 4 + a / 2, b, -s / 4 + a / 2), ((ts, 0, ts), (0, t, 0), up), dv(3, 3, 0)),    # 17
            B3((s / 4 - a / 2, b, -s / 4 - a / 2), ((a, 0, a), (0, t, 0), up), dv(1, 3, 0)),      # 18
            B3((s / 4 - a / 2 - ts, b, -s / 4 - a / 2 - ts), ((ts, 0, ts), (0, t, 0), up), dv(3, 3, 0)),  # 19
            B3((s / 4 - a / 2 - ts, 0, -s / 4 - a / 2 - ts), ((ts, 0, ts), (0, b, 0), up), dv(3, 2, 0)),  # 20
            B3((s / 4 + a / 2 + ts, 0, -s / 4 + a / 2 + ts), ((-ts, 0, -ts), (0, b, 0), dn), dv(3, 2, 0)),  # 21
            B3((s / 4 + a / 2 + ts, b, -s / 4 + a / 2 + ts), ((-ts, 0, -ts), (0, t, 0), dn), dv(3, 3, 0)),  # 22
            B3((s / 4 + a / 2, b, -s / 4 + a / 2), ((-a, 0, -a), (0, t, 0), dn), dv(1, 3, 0)),    # 23
            B3((s / 4 - a / 2, b, -s / 4 - a / 2), ((-ts, 0, -ts), (0, t, 0), dn), dv(3, 3, 0)),  # 24
            B3((s / 4 - a / 2, 0, -s / 4 - a / 2), ((-ts, 0, -ts), (0, b, 0), dn), dv(3, 2, 0)),  # 25
            P((s / 2 - b - t, 0, -s / 2 + a + b + (r + 1) * t), (0, 0, -r * t), (0, b, 0), (t, b, -t),
              (b + t, 0, -b - t)),                                                                 # 26
            T3((s / 2 - b - t, b, -s / 2 + a + b + (r + 1) * t), (0, t, 0), (t, 0, -t), (0, 0, -r * t)),  # 27
            Y((s / 2 - b - t, b, -s / 2 + a + b + t), (t, 0, -t), (0, 0, -t), (0, t, -t), (0, t, 0)),     # 28
            T3((s / 2 - b - t, b, -s / 2 + a + b), (0, t, 0), (t, 0, 0), (0, 0, -b + t)),         # 29
            P((s / 2 - b - t, 0, -s / 2 + a + b + t), (0, b, 0), *e30),                           # 30
            P((s / 2 - b - t, b, -s / 2 + a + b + t), (0, t, 0), *e30),                           # 31
            P((s / 2 - b - t, b, -s / 2 + a + t), (0, t, 0), (-r * (b + t), 0, 0),
              (-(r - 1) * h * b - t / r, 0, q1 * b + t / r), (0, 0, b)),                           # 32
            P((s / 2 - (r + 1) * (b + t), b, -s / 2), (0, t, 0), (-a + (r + 1) * (b + t), 0, 0),
              (-a + q1 * b + t / r, 0, q1 * b + q2 * t), (0, 0, a + t)),                           # 33
            P((s / 2 - a, b, -s / 2), (0, t, 0), *e34),                                            # 34
            P((s / 2 - a, 0, -s / 2), (0, b, 0), *e34),                                            # 35
            B3((s / 2 - b, b, -s / 2 + a + t), ((0, 0, -t), (-r * b, 0, 0), (-t, t, 0))),         # 36
            P((s / 2 - (r + 1) * b, b, -s / 2 + a + t), (0, 0, -t), *e37),                         # 37
            P((s / 2 - (r + 1) * b, b, -s / 2 + a), (0, 0, -a), *e37),                             # 38
            P((s / 2 - b - t, b + t, -s / 2 + a + t), (0, 0, -t), (-r * b, 0, 0),
              (-s / 4 + (2 - r) * h * b + t, s / 4 - (2 + r) * h * b - t, 0), (-s / 4 + b + t, s / 4 - b - t, 0)),  # 39
            P((s / 2 - (r + 1) * b - t, b + t, -s / 2 + a + t), (0, 0, -t), *e40),                 # 40
            P((s / 2 - (r + 1) * b - t, b + t, -s / 2 + a), (0, 0, -a), *e40),                     # 41
        ]
        ppeds = []
        for i, sp in enumerate(spec):
            kinds = self.KINDS[i]
            o = np.array(sp[1], dtype=np.float64)
            if sp[0] == "box":
                M = np.array(sp[2], dtype=np.float64).T
                dvs = sp[3]
                if dvs is None:
                    ppeds.append(Parallelepiped(o, M, np.array([-1, -1, -1]), z.copy(), kinds))
                else:
                    ppeds.append(Parallelepiped(o, M, np.array(dvs), g.copy(), kinds))
            elif sp[0] == "tri":
                M = np.array(sp[2], dtype=np.float64).T
                ppeds.append(TriangularPrism(o, M, np.array([-1, -1, -1]), z.copy(), kinds))
            else:
                mat = np.array(sp[2], dtype=np.float64).T
                cls = Prism if sp[0] == "prism" else Pyramid
                ppeds.append(cls(o, mat, -1, z.copy(), kinds))
        R = np.diag([-1.0, 1.0, 1.0])
        tr = np.array([s / 2, 0.0, -s / 2])
        pairs = [Pair(INTER, *q) for q in self.INTER_PAIRS]
        pairs += [Pair(PERI, *q, transl=tr, rot=R) for q in self.PERI_PAIRS]
        super().__init__(ppeds, pairs)

    @classmethod
    def from_cli(cls, d0, d1, d2, d3, v0, v1, v2, v3, dT):
        return cls((d0, d1, d2, d3), (v0, v1, v2, v3), dT)

    def average(self, field, cell_volumes):
        """OctetDomain::average (montecarlo/domain.cpp:1252-1280): the
        rows of `field` averaged over the cells of the vertical struts
        16-25 whose third index is 0, weighted by cell volume."""
        field = np.asarray(field)
        w = np.zeros(field.shape[1])
        col = 0
        for i, p in enumerate(self.ppeds):
            sh = p.shape()
            n = int(np.prod(sh))
            if n and i in self.AVERAGED:
                first = int(sh[0] * sh[1])  # index(2) == 0: the first layer
                w[col:col + first] = cell_volumes[col:col + first]
            col += n
        return (field * w).sum(axis=1) / w.sum()
