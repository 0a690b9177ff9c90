"""CPU: pin the oracle (C restatement + numpy orchestration) against the
reference's own outputs -- the committed golden fixtures always, and the
reference module built from its sources (oracle/_ref) when it is present."""
import sys

import numpy as np
import pytest

from oracle import oracle as O
from tests._golden import included_rows, krp_cases, load_krp, load_tree, tree_cases
from tests.conftest import REPO


@pytest.mark.parametrize("name", krp_cases())
def test_oracle_matches_golden_krp(name):
    c = load_krp(name)
    o = O.OracleKRPSampler(c["U"], c["J"], c["R"])
    samples = o.draw(c["j"], c["draws"], want_margin=True)
    rows = included_rows(c["N"], c["j"])
    # bit-exact indices; h is a product of the same rows in the same order
    assert np.array_equal(samples[rows], c["samples"][rows])
    assert np.array_equal(o.h, c["h"])
    np.testing.assert_allclose(o.weights, c["weights"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", tree_cases())
def test_oracle_matches_golden_tree(name):
    c = load_tree(name)
    n, F, R, J = (int(c[k]) for k in ("n", "F", "R", "J"))
    g = O.geometry(n, F)
    keys = ("leaf_count", "node_count", "lfill_level", "lfill_count", "total_levels",
            "nodes_upto_lfill", "nodes_before_lfill", "complete_level_offset")
    assert [g[k] for k in keys] == list(c["geometry"])
    G = O.tree_build(c["U"], F)
    np.testing.assert_allclose(G, c["G_packed"], rtol=1e-12, atol=1e-12 * np.abs(c["G_packed"]).max())
    h = c["h"].copy()
    samples = np.zeros(J, dtype=np.uint64)
    O.pt_sample(G, c["U"], F, h, np.ascontiguousarray(c["scaled_h"]), samples, c["draws"])
    assert np.array_equal(samples, c["samples"])
    assert np.array_equal(h, c["h_out"])


def test_geometry_edge_cases():
    # single leaf, power of two, one past a power of two, F = 1
    assert O.geometry(5, 8)["node_count"] == 1
    g = O.geometry(8 * 64, 8)
    assert g["leaf_count"] == 64 and g["lfill_level"] == 6 and g["node_count"] == 127
    g = O.geometry(8 * 65, 8)
    assert g["leaf_count"] == 65 and g["lfill_level"] == 6 and g["total_levels"] == 7
    g = O.geometry(13, 1)
    assert g["leaf_count"] == 13 and g["node_count"] == 25


def test_philox_known_answer():
    # Known-answer vectors published with Random123 for philox4x32_10.
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, expect in kat:
        assert O.philox4x32_10(ctr, key) == expect
    # the 53-bit uniform of counter 0 / key 0 comes from its first two words
    u = O.philox_uniforms(0, 0, 1)[0]
    assert u == (((0x6627E8D5 >> 5) << 26) | (0xE169C58D >> 6)) / 2.0**53


def _ref_module():
    ref_dir = REPO / "oracle" / "_ref"
    if not list(ref_dir.glob("ftl_ref*.so")):
        pytest.skip("reference module not built (make -C oracle ref)")
    sys.path.insert(0, str(ref_dir))
    import ftl_ref
    return ftl_ref


@pytest.mark.parametrize("N,dims,R,J,j,seed", [
    (4, [1000] * 4, 8, 10000, 5, 1),
    (3, [1001] * 3, 8, 4000, 0, 2),
    (3, [777, 64, 2000], 16, 3000, 1, 3),
    (2, [5000, 333], 32, 2000, 3, 4),
    (5, [40, 50, 60, 70, 80], 8, 3000, 2, 5),
])
def test_oracle_matches_live_reference(N, dims, R, J, j, seed):
    ftl_ref = _ref_module()
    rng = np.random.default_rng(seed)
    U = [rng.normal(size=(n, R)) for n in dims]
    draws = rng.random(2 * N * J)
    s = ftl_ref.RefSampler(U, J, R)
    ref = np.zeros((N, J), dtype=np.uint64)
    s.draw(j, ref, draws)
    hr = np.zeros((J, R))
    s.get_h(hr)
    o = O.OracleKRPSampler(U, J, R)
    out = o.draw(j, draws)
    rows = included_rows(N, j if j < N else N + 1)
    assert np.array_equal(out[rows], ref[rows])
    assert np.array_equal(o.h, hr)


def test_oracle_sketched_least_squares_residual_ratio():
    """The reference's accuracy benchmark (benchmarks/accuracy_tests_residual.py:
    21-79) as an assertion on the oracle: least squares over a 64,000-row KRP
    solved from J = 4,000 leverage samples with their weights leaves a
    residual within 1% of the exact one (the GPU test asserts the same on the
    device's samples)."""
    rng = np.random.default_rng(2024)
    N, I, R, J = 3, 40, 8, 4000
    U = [rng.normal(size=(I, R)) for _ in range(N)]
    for u in U:
        heavy = rng.choice(I, size=2, replace=False)
        u[heavy] *= 30.0
    A = np.einsum("ir,jr,kr->ijkr", *U).reshape(-1, R)
    b = A @ rng.normal(size=R) + 0.5 * rng.normal(size=A.shape[0]) * np.abs(A).mean()
    r_exact = np.linalg.norm(A @ np.linalg.lstsq(A, b, rcond=None)[0] - b)
    o = O.OracleKRPSampler(U, J, R)
    smp = o.draw(N + 1, np.random.default_rng(1).random(2 * N * J))
    rows = (smp[0].astype(np.int64) * I + smp[1].astype(np.int64)) * I + smp[2].astype(np.int64)
    sw = np.sqrt(o.weights)
    x_s = np.linalg.lstsq(sw[:, None] * A[rows], sw * b[rows], rcond=None)[0]
    assert np.linalg.norm(A @ x_s - b) / r_exact < 1.01
