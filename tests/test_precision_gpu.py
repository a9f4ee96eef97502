"""FP32 field + FP64 phases against the plain FP64 GPU solver on a chirped crystal
(the precision study at a reduced, low-gain size).  Marked gpu."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp32_meets_1e4_at_low_gain():
    from optifax_gb300 import precision as pr
    r = pr.study(pr.PrecisionCase(n_points=2 ** 12, length=1e-3, power=0.5, tau=200e-15))
    assert r["fp64"]["status"] == 0 and r["fp32"]["status"] == 0
    # with the FP64 run's decisions replayed the difference is the FP32 arithmetic alone
    assert r["fp32_replayed"]["rel_l2"] <= 1e-4, r
    assert r["fp32_replayed"]["energy_rel"] <= 1e-6, r
