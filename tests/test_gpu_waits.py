"""The error path of the bounded device-side waits: a wait that gives up sets the
filter's error word, the next call that reads the filter back reports
AMCL_ETIMEDOUT, and the filter (and the GPU context) stays usable.  The wait is
made to give up on a barrier that nothing completes, before any copy is issued, so
no copy is ever in flight when the kernel leaves; no GPU fault is involved."""

import numpy as np
import pytest

import oracle as O
from amcl3d_gb300 import _native as N
from conftest import small_grid_data

pytestmark = pytest.mark.gpu


def test_wait_probe_reports_timeout_then_recovers(amcl, ref_small):
    g = small_grid_data(ref_small)
    G = amcl.Grid3d()
    G.load_cells({"min": g.min, "max": g.max, "size": g.size, "resolution": g.res, "sensor_dev": 0.05}, g.dist,
                 g.prob)
    parts = ref_small["particles"]
    scan, ranges = ref_small["scan"], ref_small["ranges"]
    pf = amcl.ParticleFilter(seed=1)
    pf.set_option(N.OPT_WEIGHT_KERNEL, 2)  # the two-phase weighting holds the bounded waits
    pf.set_particles(parts)
    pf.set_option(N.OPT_WAIT_PROBE, 1)
    pf.update(G, scan, ranges, 0.5, 0.1, 0.0, 0.0)
    with pytest.raises(N.AmclError) as e:
        pf.getMean()
    assert e.value.status == 4  # AMCL_ETIMEDOUT
    assert b"bounded" in N.lib.amcl_last_error()
    # the probe is one-shot and the error word was cleared: the same update again is exact
    pf.set_particles(parts)
    pf.update(G, scan, ranges, 0.5, 0.1, 0.0, 0.0)
    exp, m32, _, _ = O.update_exact(parts, g, scan, ranges, 0.5, 0.1, 0.0, 0.0)
    np.testing.assert_array_equal(pf.particles(), exp)
    m = pf.getMean()
    np.testing.assert_array_equal(np.array([m.x, m.y, m.z, m.a], np.float32), m32)


def test_wait_probe_option_range(amcl):
    pf = amcl.ParticleFilter(seed=1)
    with pytest.raises(N.AmclError):
        pf.set_option(N.OPT_WAIT_PROBE, 2)
