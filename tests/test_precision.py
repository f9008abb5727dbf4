"""Double-single geometry (the default: positions, safety distances and wall roots as pairs
of floats on the FP32 pipe) against the FP64 geometry, in the CPU oracle, which each GPU
geometry matches bit for bit.  The two take different roundings at walls, so their walks
are different realisations; the test is that they sample the same temperature
distribution, by the per-cell comparison of seed ensembles used for epoch against
sequential Bjorkman & Wood."""
import numpy as np
import pytest

from tests import _cases

MRW = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)


@pytest.mark.slow
def test_double_single_and_fp64_geometry_sample_the_same_temperatures():
    """Config 1's grid (256 x 256 cells to 1e4 au, disk + Ulrich envelope, two species),
    3e4 packets, production MRW and schedule, 8 seeds of each geometry (about 85 s on 8
    cores).  Over the cells crossed >= 1e3 times per run (about 200 at this size) the z values
    of the difference of the means look like noise of a t statistic with 14 degrees of
    freedom: median |z| about 0.55, none beyond 3 sigma in this run, no mean shift.  (At 5e4
    packets and 16 seeds each: 13,794 cells, median |z| 0.70, 0.41% beyond 3 sigma.)"""
    bkw = dict(nr=256, ntheta=256)
    seeds = range(8)
    A, C = _cases.oracle_ensemble("disk_envelope", bkw, 30000, [100 + s for s in seeds], **MRW)
    B, _ = _cases.oracle_ensemble("disk_envelope", bkw, 30000, [200 + s for s in seeds],
                                  fp64_walls=True, **MRW)
    z, rel = _cases.four_sigma(A, B, C)
    assert z.size >= 150
    assert np.median(np.abs(z)) < 0.8
    assert np.mean(np.abs(z) > 4.0) < 0.02
    assert abs(np.mean(z)) < 0.3
