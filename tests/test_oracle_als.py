"""CPU: the numpy ALS oracle (oracle/oracle.py: OracleALS) against the
reference's ALS outputs -- the committed golden fixtures, and the live
reference module when it is built."""
import sys

import numpy as np
import pytest

from oracle import oracle as O
from tests._golden import als_cases, load_als
from tests.conftest import REPO


@pytest.mark.parametrize("name", als_cases())
def test_oracle_als_matches_golden(name):
    c = load_als(name)
    o = O.OracleALS(c["U0"], c["sigma0"], c["idx"], c["vals"], c["J"], c["dims"])
    for u, upd in enumerate(c["updates"]):
        j = upd["j"]
        o.update(j, upd["draws"])
        rows = [k for k in range(c["N"]) if k != j]
        assert np.array_equal(o.last_samples[rows], upd["samples"][rows]), f"update {u}"
        np.testing.assert_allclose(o.U[j], upd["U"], rtol=0, atol=1e-12 * np.abs(upd["U"]).max())
        np.testing.assert_allclose(o.sigma, upd["sigma"], rtol=1e-12)
        if (u + 1) % c["N"] == 0:
            np.testing.assert_allclose(o.residual_normsq(), c["resid"][u // c["N"]], rtol=1e-11)


def test_oracle_als_matches_live_reference():
    ref_dir = REPO / "oracle" / "_ref"
    if not list(ref_dir.glob("ftl_ref*.so")):
        pytest.skip("reference module not built (make -C oracle ref)")
    sys.path.insert(0, str(ref_dir))
    import ftl_ref
    rng = np.random.default_rng(77)
    dims, N, R, J, nnz = [25, 35, 45], 3, 6, 350, 1800
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = rng.random(nnz) + 0.5
    U = [rng.normal(size=(d, R)) for d in dims]
    lr = ftl_ref.LowRankTensor(R, U)
    lr.renormalize_columns(-1)
    sig = np.zeros(R)
    lr.get_sigma(sig, -1)
    o = O.OracleALS([u.copy() for u in U], sig, idx, vals, J, dims)
    sp = ftl_ref.SparseTensor(idx, vals, "sort")
    als = ftl_ref.InjectedALS(lr, sp)
    als.initialize_ds_als(J)
    for j in [0, 1, 2, 0, 1, 2]:
        d = rng.random(2 * N * J)
        als.set_draws(d)
        als.execute_ds_als_update(j, True, True)
        o.update(j, d)
        np.testing.assert_allclose(o.U[j], U[j], rtol=0, atol=1e-12 * np.abs(U[j]).max())
    s2 = np.zeros(R)
    lr.get_sigma(s2, -1)
    np.testing.assert_allclose(o.residual_normsq(), sp.compute_residual_normsq(s2, U), rtol=1e-11)
