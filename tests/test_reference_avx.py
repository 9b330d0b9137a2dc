"""Direct comparison with the reference's own CPU code, compiled from its
sources into oracle/_ref; runs only where that build exists (x86_64 hosts
with the reference tree)."""
import numpy as np
import pytest

from conftest import rel_vec_err, rows_equal
from nbody6ppgpu_gb300 import ics
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.RefAVX.available(), reason="reference AVX build absent")


@pytest.mark.parametrize("seed,n,target,m_flag", [(11, 1000, 40.0, 0), (12, 777, 25.0, 1)])
def test_fresh_inputs_against_reference(seed, n, target, m_flag):
    c = ics.plummer(n, seed=seed, masses="kroupa" if m_flag else "equal", nb_target=target)
    h2 = c.h2(m_flag, float(c.m.mean()))
    ref = O.RefAVX(4096)
    ref.send(c.m, c.x, c.v)
    ra, rj, rp, rl = ref.regf(h2, c.dtr, c.x, c.v, 300, 299, m_flag)
    ref.close()
    oa, oj, op, ol = O.regf_fp64(c.m, c.x, c.v, h2, c.dtr, c.x, c.v, 300, 299, m_flag)
    # the FP32 reference and the FP64 oracle may disagree only for pairs whose
    # criterion lies within the reference's own FP32 rounding of it
    bad = rows_equal(rl, ol)
    assert len(bad) <= max(1, n // 500)
    assert np.percentile(rel_vec_err(ra, oa), 99) < 5e-6
