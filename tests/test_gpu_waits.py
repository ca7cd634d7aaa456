"""The asynchronous waits of the kernels (the mbarrier waits of the static
kernel's bulk-copy stream) are bounded: a wait that nothing completes gives
up on its own with the timeout status the host reads, and the device stays
usable. No GPU fault, trap or hang is involved: the wait's own deadline ends
it."""

import ctypes as C

import pytest

import montecarlocpp_gb300 as M
from montecarlocpp_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_wait_that_nothing_completes_gives_up(gmat):
    st, waited = C.c_uint(0), C.c_double(0.0)
    _lib.check(_lib.lib().mc_check_bounded_wait(20.0, C.byref(st), C.byref(waited)))
    assert st.value & 8, "the wait did not report giving up"
    assert 20.0 <= waited.value < 2000.0
    # the context still works: a per-step solve (the bulk-copy stream) runs clean
    P = M.MultiProblem(gmat, M.FilmDomain.from_cli(1e-7, 1e-7, 10), 2000, 10**6)
    P.solve(dt=0.5e-12, nsteps=40, precision=32, steps_per_launch=1, schedule=1, seed=2)
    assert P.stats["status"] == 0 and P.stats["phonon_steps"] == 40 * P.stats["nemit"]
