"""Grid sizes the solver accepts (no GPU: the check is in the constructor).

Axis lengths 2^a and 3 * 2^a: x in [2, 2048] (3 * 2^a up to 384), y and z in [1, 1024]
(3 * 2^a up to 192).  Odd lengths and other factors (5, 7, ...) are refused with
CUPSSGB_ERR_UNSUPPORTED.
"""
import pytest


@pytest.mark.parametrize("shape", [(96, 96, 96), (192, 192, 192), (384, 192, 1), (6, 1, 1), (2048, 1024, 1),
                                   (12, 6, 6), (96, 64, 48), (1024, 1, 1)])
def test_accepted(built_lib, shape):
    from cupss_gb300.api import Solver
    s = Solver(*shape)
    s.close()


@pytest.mark.parametrize("shape", [(80, 80, 1), (96, 384, 1), (768, 1, 1), (3, 1, 1), (9, 9, 1), (64, 64, 320),
                                   (100, 1, 1), (4096, 1, 1), (1, 1, 1), (64, 3, 1)])
def test_refused(built_lib, shape):
    from cupss_gb300.api import Solver
    from cupss_gb300.capi import CupssError
    with pytest.raises(CupssError) as ex:
        Solver(*shape)
    assert ex.value.code == -3
