"""The batch at its configuration size: 256 independent cases (128 lid
cavities of 2k-60k cells and 128 porous squares of 10k-120k cells with 20-200
obstacles, Re 50-400 through tau), about 12.7M cells in one packed launch per
kernel, match the C oracle case by case, bit for bit (cell pdfs, node pdfs),
after 5 steps."""
import os

import numpy as np
import pytest

import oracle_c as OC
import oracle_np as ON

pytestmark = pytest.mark.gpu


def test_config_size_batch_bitwise():
    from fvdbm_jax_gb300 import Batch
    from fvdbm_jax_gb300 import cases as CS
    suite, desc = CS.batch_suite(seed=0, workers=min(16, os.cpu_count() or 1))
    assert len(suite) == 256 and sum(d["cells"] for d in desc) > 10_000_000
    b = Batch([(c, f, n) for _, c, f, n in suite])
    b.init()
    b.step(5)
    st = b.state()
    for s, (dyn, c, f, n) in enumerate(suite):
        got = b.case_state(s, st)
        geo, st0 = ON.geo_from_containers(c, f, n), ON.state_from_containers(c, n)
        orc = OC.step(geo, st0, dyn.inv_tau, dyn.dt32, 5)
        assert np.array_equal(got["pdf"], orc["cells_pdf"]), (s, desc[s])
        assert np.array_equal(got["node_pdf"].reshape(orc["nodes_pdf"].shape), orc["nodes_pdf"]), (s, desc[s])
    b.close()
