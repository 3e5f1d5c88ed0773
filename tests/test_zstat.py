"""The calibrated z-test (zstat.ztest) on the CPU, oracle images only: an
independent oracle image passes; images with planted mistakes (a 3% bias
over the frame, one 8x8 block 50% too bright in one channel) fail. At 64
samples per pixel of the 32x32 Cornell box these are about the smallest
mistakes of either kind the test detects.""" 
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from zstat import oracle_ref_and_null, ztest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
S, N = 64, 1024


@pytest.fixture(scope="module")
def cornell():
    o = Oracle(os.path.join(GOLDEN, "scenes", "cornell", "renderJob.json"))
    o.set_seed(777)
    w, h = o.info()["width"], o.info()["height"]
    t = o.render(0, S, 0, 0, w, h)
    ref = oracle_ref_and_null(o, S, N, 0, 0, w, h)
    o.close()
    return t["color"], t["color_sq"], ref


def test_independent_oracle_image_passes(cornell):
    ts, ts2, (cs, cs2, nulls) = cornell
    ztest("oracle vs oracle", ts, ts2, S, cs, cs2, N, nulls)


def test_planted_bias_fails(cornell):
    ts, ts2, (cs, cs2, nulls) = cornell
    k = 1.03
    with pytest.raises(AssertionError):
        ztest("3% bias", ts * k, ts2 * k * k, S, cs, cs2, N, nulls)


def test_planted_region_fails(cornell):
    ts, ts2, (cs, cs2, nulls) = cornell
    bad, bad2 = ts.copy(), ts2.copy()
    bad[8:16, 8:16, 1] *= 1.5           # green channel of one 8x8 block 50% too bright
    bad2[8:16, 8:16, 1] *= 1.5 ** 2
    with pytest.raises(AssertionError):
        ztest("bright block", bad, bad2, S, cs, cs2, N, nulls)
