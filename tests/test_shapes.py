"""Subdomains other than the Parallelepiped on the CPU: the oracle's
restatement of TriangularPrism, Tetrahedron, Prism<N> and Pyramid<N>
(montecarlo/subdomain.h:207-640, montecarlo/subdomain.cpp:283-441) and of
the Triangle / Polygon faces (montecarlo/boundary.cpp:154-258), checked
against the reference's formulas, and the library's domain image checked
against the oracle's. No GPU needed."""

import numpy as np
import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import domains as D
from oracle import oracle as O

import shape_cases as SC


def _tri_prism(div, nf_cls=D.TriangularPrism, nf=5):
    return nf_cls(np.zeros(3), np.diag([1e-7, 2e-7, 1e-7]), np.array(div), np.array([-1e6, 0, 0]), (D.SPEC,) * nf)


@pytest.mark.parametrize("div", [(10, 10, 0), (10, 0, 0), (4, 6, 3), (1, 1, 1)])
def test_cell_volumes_follow_the_reference(div):
    """TriangularPrismImpl / TetrahedronImpl::cellVol as the reference
    computes them: full cells vol / prod(shape), cut cells from the corner
    formula, cells outside 0; they add up to vol / 2 and vol / 6. The
    library's cell volumes are the oracle's, bit for bit."""
    for cls, nf, frac in ((D.TriangularPrism, 5, 0.5), (D.Tetrahedron, 4, 1.0 / 6.0)):
        p = _tri_prism(div, cls, nf)
        dom = D.Domain([p], [])
        cv = O.ODomain(dom).cell_volumes()
        assert cv.sum() == pytest.approx(frac * p.vol(), rel=1e-12)
        shape = np.maximum(np.array(div), 1)
        # cell (0, 0, 0) is full unless the grid is one cell across
        if (shape[:2] > 2).all():
            assert cv[0] == pytest.approx(p.vol() / np.prod(shape), rel=1e-14)
        h = M.problem.DomainHandle(dom)
        assert np.array_equal(h.cell_volumes(), cv)


@pytest.mark.parametrize("name", list(SC.cases()))
def test_emitted_positions_lie_in_the_subdomain(name):
    dom = SC.cases()[name][0]
    od = O.ODomain(dom)
    w, sd, fc = od.emitters()
    assert len(w) > 0 and (w > 0).all()
    for e in range(len(w)):
        x = od.draw_positions(e, 3, 1500)
        assert all(od.is_inside(sd[e], xi) for xi in x)


def test_triangle_and_polygon_face_draws_are_uniform():
    """Triangle::drawPos folds the unit square onto the triangle and
    Polygon<N>::drawPos picks a triangle by area first: the mean of many
    draws is the face's centroid."""
    dom = SC.pyr5()
    od = O.ODomain(dom)
    w, sd, fc = od.emitters()
    p = dom.ppeds[0]
    c = p.columns()
    base = np.array([np.zeros(3)] + [c[:, i] for i in range(1, c.shape[1])])
    # centroid of the pentagon (o, c1 .. c4) by triangle fan from o
    tri = [(base[0], base[i], base[i + 1]) for i in range(1, len(base) - 1)]
    area = np.array([np.linalg.norm(np.cross(b - a, cc - a)) / 2 for a, b, cc in tri])
    cen = sum(ar * (a + b + cc) / 3 for ar, (a, b, cc) in zip(area, tri)) / area.sum()
    x = od.draw_positions(fc.index(0), 11, 200000)
    assert np.allclose(x.mean(axis=0), cen, atol=2e-10)
    # face 3 = side 2: Triangle(c0 - c2, c3 - c2) at o + c2, i.e. the
    # triangle (o + c2, apex, o + c3)
    x = od.draw_positions(fc.index(3), 12, 200000)
    a, b, cc = c[:, 2], c[:, 0], c[:, 3]
    assert np.allclose(x.mean(axis=0), (a + b + cc) / 3, atol=2e-10)


def test_prism_and_pyramid_volumes_follow_the_reference():
    """PrismImpl / PyramidImpl::volume sum col(i) x col(i+1) . col(0) over
    i < N - 2 and drawPos picks sub-volume ind with columns (ind + 1,
    ind + 2, 0): the first weight is 0, so no position lands in the first
    sub-volume. Both kept as the reference has them."""
    dom = D.PyrDomain.from_cli(1e-7, 1e-7)
    od = O.ODomain(dom)
    p = dom.ppeds[0]
    c = p.columns()
    assert od.sdom_volume(0) == pytest.approx(np.dot(np.cross(c[:, 1], c[:, 2]), c[:, 0]) / 6, rel=1e-14)
    x = od.draw_positions(0, 5, 4000)
    # sub-volume 1 = tetrahedron (o, c2, c3, c0): all points have
    # barycentric coordinates >= 0 in it
    T = np.stack([c[:, 2], c[:, 3], c[:, 0]], axis=1)
    lam = np.linalg.solve(T, x.T)
    assert (lam > -1e-12).all() and (lam.sum(axis=0) < 1 + 1e-12).all()


def test_library_refuses_what_the_kernels_do_not_take():
    """HexDomain's Prism<6> (eight faces) and JctDomain (one Inter face
    paired with two others) take a continuation slot each; more than 64
    slots in all is MC_ERR_UNSUPPORTED, which the oracle does not limit."""
    hexp = D.HexDomain.from_cli(1e-7, 5e-8).ppeds[0]
    ppeds, pairs = [], []
    for i in range(33):
        ppeds.append(D.Prism(hexp.o + np.array([0.0, 3e-7 * i, 0.0]), hexp.mat, 0, hexp.gradT, hexp.kinds))
        pairs.append(D.Pair(D.PERI, i, 0, i, 1, np.array([1e-7, 0.0, 0.0])))
    dom = D.Domain(ppeds, pairs)
    O.ODomain(dom)
    with pytest.raises(M._lib.McError) as e:
        M.problem.DomainHandle(dom)
    assert e.value.code == -4
    for d in (D.HexDomain.from_cli(1e-7, 5e-8), D.JctDomain.from_cli(1e-7, 1e-7)):
        assert M.problem.DomainHandle(d).cols == O.ODomain(d).cols


def test_library_and_oracle_agree_on_columns_and_weights():
    for name, (dom, *_rest) in SC.cases().items():
        od = O.ODomain(dom)
        h = M.problem.DomainHandle(dom)
        assert h.cols == od.cols, name
        cv = od.cell_volumes()
        assert np.array_equal(h.cell_volumes(), cv), name


def test_octet_domain_assembles_and_averages():
    """OctetDomain: 42 subdomains whose Inter and Peri pairs pass the
    makePair checks (the library refuses mismatched planes); its field
    columns are the ten struts' cells, and average() weights the first cell
    layer of struts 16-25 by cell volume (montecarlo/domain.cpp:1252-1280)."""
    dom = D.OctetDomain((3e-7, 5e-8, 5e-8, 5e-9), (4, 3, 2, 2), 1e-1)
    assert len(dom.ppeds) == 42
    h = M.problem.DomainHandle(dom)
    od = O.ODomain(dom)
    assert h.cols == od.cols == dom.cols() == 176
    cv = h.cell_volumes()
    assert np.array_equal(cv, od.cell_volumes())
    f = np.vstack([np.ones(h.cols), np.arange(h.cols, dtype=float)])
    avg = dom.average(f, cv)
    assert avg[0] == pytest.approx(1.0)
    # by hand: the first layer of each strut
    num = den = 0.0
    col = 0
    for i, p in enumerate(dom.ppeds):
        n = int(np.prod(p.shape()))
        if n and 16 <= i < 26:
            k = int(p.shape()[0] * p.shape()[1])
            num += float((cv[col:col + k] * np.arange(col, col + k)).sum())
            den += float(cv[col:col + k].sum())
        col += n
    assert avg[1] == pytest.approx(num / den)


def test_makepair_checks():
    """makePair refuses Inter faces whose planes differ (montecarlo/
    boundary.cpp:363-368) and Peri maps that do not carry one face onto the
    other (boundary.cpp:527-535)."""
    box = lambda o: D._pped(o, (1e-7, 1e-7, 1e-7), (0, 0, 0), (0, 0, 0), (D.INTER, D.SPEC, D.SPEC, D.SPEC, D.SPEC, D.SPEC))
    box2 = lambda o: D._pped(o, (1e-7, 1e-7, 1e-7), (0, 0, 0), (0, 0, 0), (D.SPEC, D.SPEC, D.SPEC, D.INTER, D.SPEC, D.SPEC))
    ok = D.Domain([box((1e-7, 0, 0)), box2((0, 0, 0))], [D.Pair(D.INTER, 0, 0, 1, 3)])
    M.problem.DomainHandle(ok)
    gap = D.Domain([box((1.1e-7, 0, 0)), box2((0, 0, 0))], [D.Pair(D.INTER, 0, 0, 1, 3)])
    with pytest.raises(M._lib.McError):
        M.problem.DomainHandle(gap)
    film = D.FilmDomain.from_cli(1e-7, 1e-7, 4)
    film.pairs[0].transl = np.array([1.2e-7, 0.0, 0.0])
    with pytest.raises(M._lib.McError):
        M.problem.DomainHandle(film)


def _random_shapes(rng):
    """Random convex subdomains of each shape with positive volume."""
    out = []
    for _ in range(4):
        M = np.diag(rng.uniform(0.5e-7, 2e-7, 3)) + rng.uniform(-2e-8, 2e-8, (3, 3))
        div = rng.integers(1, 5, 3)
        out.append(D.TriangularPrism(rng.uniform(-1e-7, 1e-7, 3), M, div, np.zeros(3), (D.SPEC,) * 5))
        out.append(D.Tetrahedron(rng.uniform(-1e-7, 1e-7, 3), M, div, np.zeros(3), (D.SPEC,) * 4))
        # a convex base polygon in the y-z plane, counter-clockwise, and an
        # axis or apex along +x
        n = int(rng.integers(4, 7))
        ang = np.linspace(0, 2 * np.pi, n, endpoint=False) + rng.uniform(0, 0.3)
        pts = np.stack([np.zeros(n), np.cos(ang), np.sin(ang)], axis=1) * 5e-8
        base = pts[1:] - pts[0]
        axis = np.array([1e-7, *rng.uniform(-2e-8, 2e-8, 2)])
        mat = np.vstack([axis, base]).T
        out.append(D.Prism(pts[0], mat, int(rng.integers(-1, 1)), np.zeros(3), (D.SPEC,) * (n + 2)))
        apex = pts.mean(axis=0) - pts[0] + np.array([1e-7, 0, 0])
        out.append(D.Pyramid(pts[0], np.vstack([apex, base]).T, 0, np.zeros(3), (D.SPEC,) * (n + 1)))
    return out


def test_random_shapes_library_matches_oracle():
    """Random TriangularPrisms, Tetrahedra, Prisms and Pyramids: the
    library and the oracle give the same columns and cell volumes, and the
    oracle's emission positions (a gradient makes every shape a volume
    emitter) lie inside."""
    rng = np.random.default_rng(11)
    for p in _random_shapes(rng):
        p.gradT = np.array([-1e6, 0.0, 0.0])
        dom = D.Domain([p], [])
        od = O.ODomain(dom)
        h = M.problem.DomainHandle(dom)
        assert h.cols == od.cols
        assert np.array_equal(h.cell_volumes(), od.cell_volumes())
        w, sd, fc = od.emitters()
        assert len(w) == 1 and fc[0] == -1
        x = od.draw_positions(0, 5, 300)
        assert all(od.is_inside(0, xi) for xi in x), type(p).__name__
