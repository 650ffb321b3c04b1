"""The device-side bounded wait's error path, exercised without a GPU fault.

The multigrid's single-CTA tail stages its first level into shared memory with TMA bulk copies completed on
an mbarrier, and waits for them at most a bounded number of polls.  fire_sim_set_tail_wait_limit(0) makes
that first wait give up at once on a healthy GPU: the kernel records the timeout in a device flag, waits
again (at the full bound) for the copies still in flight, and returns without running the cycle.  The host
must then see FIRE_ERR_CUDA with the timeout message from fire_sim_sync, the flag must be cleared by that
report, the context must stay usable, and steps with the normal bound must run clean again.  At 48x96x48 the
tail starts at 12x24x12 (3456 cells, 16-byte aligned arrays), so it takes the bulk-copy path.
"""
import numpy as np
import pytest

import fire_cases as FC
import fire_sim as F

pytestmark = pytest.mark.gpu


def test_tail_wait_timeout_is_reported_and_recoverable():
    sim = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=F.build_campfire(7), vcycles=2)
    dt = FC.C1["dt"]
    sim.step(dt, 3)
    sim.sync()
    ref = F.FireSim(res=FC.C1["res"], size=FC.C1["size"], logs=F.build_campfire(7), vcycles=2)
    ref.step(dt, 3)
    ref.sync()
    sim.set_tail_wait_limit(0)
    sim.step(dt, 1)
    with pytest.raises(F.FireError) as ei:
        sim.sync()
    assert ei.value.code == 3 and "timed out" in str(ei.value), ei.value
    sim.sync()                          # the report cleared the flag; the context is still usable
    assert np.isfinite(sim.download("vel")).all()
    # the cycle was skipped, so this step's pressure differs from a clean step's
    ref.step(dt, 1)
    ref.sync()
    assert not np.array_equal(sim.level(0, "p"), ref.level(0, "p"))
    sim.set_tail_wait_limit(1 << 22)
    sim.step(dt, 2)
    sim.sync()                          # clean again with the normal bound
    assert np.isfinite(sim.download("S")).all()
    sim.close()
    ref.close()
