"""The deterministic epoch form of Bjorkman & Wood against the classic sequential form
(the reference algorithm: every absorption reads the running temperature), both in the
CPU oracle: over 8 seeds each, the per-cell mean temperatures agree within 4 sigma of
the seed-to-seed scatter in every heated cell crossed >= 1e3 times per run, and the
differences are consistent with that scatter (median |z| < 1; pure noise gives 0.67).
At 1e6 packets per run (too slow for this suite) the median relative difference of the
two forms is 0.65%."""
import numpy as np

from pdspy_gb300 import workloads
from tests import _cases

MRW = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)


def test_epoch_and_sequential_agree_within_four_sigma():
    m = workloads.small_disk(nr=24, ntheta=24, mass=1e-4, g=0.6)
    E, S, C = [], [], 0
    for seed in range(8):
        a = _cases.run_oracle(m, 20000, seed=seed, crossings=True, **MRW)
        b = _cases.run_oracle(m, 20000, seed=100 + seed, sequential=True, **MRW)
        E.append(a["temperature"][0])
        S.append(b["temperature"][0])
        C = C + a["crossings"]
    E, S = np.array(E), np.array(S)
    me, ms = E.mean(0), S.mean(0)
    sigma = np.sqrt(E.var(0, ddof=1) / 8 + S.var(0, ddof=1) / 8)
    sel = (C / 8 >= 1000) & (ms > 0) & (me > 0)
    assert sel.sum() >= 50
    z = np.abs(me - ms)[sel] / sigma[sel]
    assert np.all(z < 4.0), z.max()
    assert np.median(z) < 1.0
