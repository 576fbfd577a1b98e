"""Failure handling without a GPU fault: every device loop is bounded and reports a status the
host reads.  With the round cap at 0 every unit of every kernel family (plain, shared-memory,
frontier) stops at once; the call returns FBC_ERR_ITER_LIMIT and the library stays usable."""
import numpy as np
import pytest

import graphs
import oracle
from test_gpu_parity import TOL_FP64, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sched,warp_max_n", [(0, 4096), (1, 4096), (1, 0)])
def test_round_cap_reports_and_recovers(fg, sched, warp_max_n):
    el = graphs.WORKLOADS["grid32"]()
    g = fg.Graph.from_edgelist(el)
    old = (fg.get_option("iter_mult"), fg.get_option("warp_max_n"))
    fg.set_option("warp_max_n", warp_max_n)  # 4096: the shared-memory kernel, 0: the frontier kernel
    try:
        fg.set_option("iter_mult", 0)
        with pytest.raises(fg.FbcError) as e:
            fg.exact_bc(g, fg.FP64, sched)
        assert e.value.code == fg.FBC_ERR_ITER_LIMIT
        fg.set_option("iter_mult", old[0])
        ref = oracle.exact_bc(oracle.CSR.from_edgelist(el))
        assert rel_err(fg.exact_bc(g, fg.FP64, sched), ref) <= TOL_FP64
    finally:
        fg.set_option("iter_mult", old[0])
        fg.set_option("warp_max_n", old[1])
