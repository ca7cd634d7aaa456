"""Test domains with subdomains other than the Parallelepiped, built only
from the reference's constructors (montecarlo/subdomain.h:207-640) and
makePair, plus the reference's own Pyr, Tee and Tube domains."""

import numpy as np

from montecarlocpp_gb300 import domains as D


def wedge():
    """TriangularPrism, 1-D field along its length: isothermal triangles at
    both ends (Triangle emission), diffuse and specular sides, a skew
    diagonal face."""
    p = D.TriangularPrism(np.zeros(3), np.diag([1e-7, 1.2e-7, 2e-7]), np.array([0, 0, 20]), np.zeros(3),
                          (D.DIFF, D.SPEC, D.ISOT, D.DIFF, D.ISOT), (0.0, 0.0, 1.0, 0.0, -1.0))
    return D.Domain([p], [])


def tet():
    """Tetrahedron with a sheared matrix, a 3-D field (cells outside the
    shape have zero volume) and a volumetric gradient."""
    M = np.array([[1e-7, 2e-8, 0.0], [0.0, 1e-7, 1e-8], [0.0, 0.0, 1e-7]])
    p = D.Tetrahedron(np.array([1e-8, 0.0, 0.0]), M, np.array([4, 4, 4]), np.array([-1e6, 2e5, 0.0]),
                      (D.SPEC, D.DIFF, D.SPEC, D.DIFF))
    return D.Domain([p], [])


def prism4():
    """Prism<4>: quadrilateral rod along x, periodic end caps (Polygon<4>
    faces), diffuse and specular sides, volumetric gradient along x."""
    mat = np.array([[1e-7, 0, 0], [0, 1e-7, 0], [0, 1.2e-7, 8e-8], [0, 0, 1e-7]]).T
    p = D.Prism(np.zeros(3), mat, 0, np.array([-1e6, 0.0, 0.0]),
                (D.PERI, D.PERI, D.DIFF, D.SPEC, D.DIFF, D.SPEC))
    return D.Domain([p], [D.Pair(D.PERI, 0, 0, 0, 1, np.array([1e-7, 0.0, 0.0]))])


def pyr5():
    """Pyramid<5>: pentagonal base held at +1 (Polygon<5> emission), one
    side at -1 (Triangle emission), diffuse and specular sides."""
    mat = np.array([[5e-8, 5e-8, 1e-7], [1e-7, 0, 0], [1.3e-7, 7e-8, 0], [6e-8, 1.2e-7, 0],
                    [-2e-8, 8e-8, 0]]).T
    p = D.Pyramid(np.zeros(3), mat, 0, np.zeros(3), (D.ISOT, D.DIFF, D.SPEC, D.ISOT, D.DIFF, D.SPEC),
                  (1.0, 0.0, 0.0, -1.0, 0.0, 0.0))
    return D.Domain([p], [])


def cases():
    """name -> (domain, problem kind, nemit, dt, nsteps)"""
    import montecarlocpp_gb300 as M
    return {
        "wedge": (wedge(), M.MULTI, 1500, 1e-12, 400),
        "tet": (tet(), M.MULTI, 1500, 0.5e-12, 400),
        "prism4": (prism4(), M.MULTI, 1500, 0.5e-12, 400),
        "pyr5": (pyr5(), M.TEMP, 1500, 1e-12, 400),
        "pyr": (D.PyrDomain.from_cli(1e-7, 1e-7), M.MULTI, 1500, 0.5e-12, 400),
        "tee": (D.TeeDomain.from_cli(5e-8, 3e-8, 4), M.MULTI, 1500, 0.5e-12, 400),
        "tube": (D.TubeDomain.from_cli(1e-7, 5e-8, 2e-8, 5, 3), M.MULTI, 1500, 0.5e-12, 400),
        "hex": (D.HexDomain.from_cli(1e-7, 4e-8), M.MULTI, 1500, 0.5e-12, 400),
        "jct": (D.JctDomain((5e-8, 5e-8, 5e-8, 4e-8), (4, 3, 3, 0), 1e-1), M.MULTI, 1500, 0.5e-12, 400),
        "octet": (D.OctetDomain((3e-7, 5e-8, 5e-8, 5e-9), (4, 3, 2, 2), 1e-1), M.MULTI, 2000, 0.5e-12, 400),
    }
