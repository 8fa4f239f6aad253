"""The oracle's operation counter (oracle/op_count.cpp: the oracle source
compiled with a counting number type) builds and counts the reference
scheme's arithmetic: the numerator of the benchmark's roofline figures."""
import pytest

from oracle import oracle
from reprobus_gb300 import inputs


def test_op_counter_counts_the_reference_step():
    case = inputs.make_case("grid", seed=3, nlon=4, nlat=3, nivbas=94)
    one = oracle.op_counts(case, [2], niter=1)
    five = oracle.op_counts(case, [2], niter=5)
    assert one["cells"] == five["cells"] == 4 * 94
    # the rate stage runs once per step, the passes niter times
    for k in ("add", "mul", "div"):
        assert five[k] > one[k] > 0, k
    assert five["exp"] == pytest.approx(one["exp"])  # exponentials only in the rate stage
    per_pass = (five["flops"] - one["flops"]) / 4
    assert 500 < per_pass < 5000
    assert five["transcendentals"] > 100
