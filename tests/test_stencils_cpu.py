"""Caller-built stencils (pdds_stencils_set) on a host-only context.

Every knot of a built layout handed back with its own stencil (the
reference's per-knot Stencil::Init input) rebuilds the same G structure:
the same CSR columns and the same stencils.  Malformed stencils are refused
with PDDS_ERR_INVALID.  No GPU is needed: a context created for device -1
builds layouts on the host only.
"""
import numpy as np
import pytest

import pdds_gb300 as P
from pdds_gb300.config import fac_rule


def _host(sw, ne, nsub, nnode):
    return P.PDDSparseGM(sw, ne, nsub, nnode, fac_rule(ne[0] - sw[0], nsub, nnode), device=-1)


@pytest.mark.parametrize("sw,ne,nsub,nnode", [((-1.0, -1.0), (1.0, 1.0), 4, 11), ((0.0, 0.0), (1.0, 1.0), 3, 6)])
def test_layout_rebuilt_from_its_stencils(sw, ne, nsub, nnode):
    with _host(sw, ne, nsub, nnode) as pd:
        sts = [P.Stencil.of_knot(pd, k) for k in range(pd.K)]
        with P.PDDSparseGM.from_stencils((sw[0], sw[1], ne[0], ne[1]), pd.x, pd.y, sts, device=-1) as q:
            assert q.K == pd.K
            assert q.layout_info["nboundary"] == pd.layout_info["nboundary"]
            np.testing.assert_array_equal(q.row_ptr, pd.row_ptr)
            np.testing.assert_array_equal(q.col, pd.col)
            for k in range(0, pd.K, 7):
                r1, _, s1 = pd.stencil(k)
                r2, _, s2 = q.stencil(k)
                np.testing.assert_array_equal(r1, r2)
                for a, b in zip(s1, s2):
                    np.testing.assert_array_equal(a, b)
            # shared sides and shapes are found again
            assert q.layout_info["nshapes"] <= pd.layout_info["nshapes"] + 4


def test_init_rule_drops_consecutive_repeats_and_keeps_last_position():
    st = P.Stencil((0.0, 0.0, 1.0, 1.0), (0.0, 0.0, 1.0, 1.0))
    st.Init({"N": [5, 5, 6, 7]}, {"N": [0.1, 0.2, 0.5, 0.9]}, {"N": [1.0, 1.0, 1.0, 1.0]}, (0.0, 0.0, 1.0, 1.0))
    st.Compute_ipsi(0.3)
    with P.PDDSparseGM.from_stencils((-1.0, -1.0, 2.0, 2.0), [0.5], [0.5], [st], device=-1) as q:
        assert q.nnz == 3
        np.testing.assert_array_equal(q.col, [5, 6, 7])
        r, kinds, sides = q.stencil(0)
        np.testing.assert_array_equal(sides[0], [5, 6, 7])


@pytest.mark.parametrize("bad", ["off_line", "order", "c2", "rect"])
def test_malformed_stencils_are_refused(bad):
    st = P.Stencil((0.0, 0.0, 1.0, 1.0), (0.0, 0.0, 1.0, 1.0))
    xs, ys = [0.1, 0.5, 0.9], [1.0, 1.0, 1.0]
    if bad == "off_line":
        ys = [1.0, 0.9, 1.0]
    if bad == "order":
        xs = [0.5, 0.1, 0.9]
    st.Init({"N": [1, 2, 3]}, {"N": xs}, {"N": ys}, (0.0, 0.0, 1.0, 1.0) if bad != "rect" else (1.0, 0.0, 0.0, 1.0))
    st.Compute_ipsi(0.3 if bad != "c2" else 0.0)
    with pytest.raises(P.PDDSError) as e:
        P.PDDSparseGM.from_stencils((-1.0, -1.0, 2.0, 2.0), [0.5], [0.5], [st], device=-1)
    assert "INVALID" in str(e.value)
