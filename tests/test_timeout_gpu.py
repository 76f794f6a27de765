"""A device-side wait that runs out ends with a status, not a hang."""
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out(gme_ctx):
    st = gme_ctx.debug_wait_timeout(20_000_000)   # 20 ms on a flag nothing sets
    assert st == 4                                 # GME_ERR_TIMEOUT
    # the context is still usable afterwards
    r = gme_ctx.align(0, [1, 2, 3], [1, 3])
    assert r.score == 2
