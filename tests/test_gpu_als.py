"""GPU parity of the randomized CP-ALS path against the reference's ALS
(golden fixtures recorded from cpp_ext/als.hpp with injected uniforms) and
the numpy ALS oracle.

Tolerances: sampled indices identical (the trees are rebuilt from factors
that agree to ~1e-13, so only near-ties could flip; none are allowed here);
updated factors within 1e-9 of the largest entry; sigma and residuals within
1e-9 relative; the CP fit (1 - ||X - model|| / ||X||) within 1e-6 relative,
the target for the fit.  FP32 sampling: residual within 1e-3 relative of the
FP64 trajectory.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests._golden import als_cases, load_als

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def _setup(ftl, c, precision="fp64"):
    U = [np.ascontiguousarray(u.copy()) for u in c["U0"]]
    lr = ftl.LowRankTensor(c["R"], U)
    lr.set_sigma(c["sigma0"])
    sp = ftl.SparseTensor(c["idx"], c["vals"], "sort", dims=c["dims"])
    als = ftl.ALS(lr, sp)
    als.initialize_ds_als(c["J"], "efficient", precision=precision)
    return U, lr, sp, als


@pytest.mark.parametrize("name", als_cases())
def test_gpu_als_matches_reference_golden(ftl, name):
    c = load_als(name)
    U, lr, sp, als = _setup(ftl, c)
    assert abs(sp.get_normsq() - c["normsq"]) <= 1e-12 * c["normsq"]
    N = c["N"]
    for u, upd in enumerate(c["updates"]):
        j = upd["j"]
        als.execute_ds_als_update(j, True, True, draws=upd["draws"])
        samples = als.sampler.samples_dev.cpu().numpy().view(np.uint64)
        rows = [k for k in range(N) if k != j]
        assert np.array_equal(samples[rows], upd["samples"][rows]), f"update {u}: samples differ"
        # the host array is updated in place, like the reference's numpy factors
        np.testing.assert_allclose(U[j], upd["U"], rtol=0, atol=1e-9 * np.abs(upd["U"]).max())
        np.testing.assert_allclose(lr.sigma, upd["sigma"], rtol=1e-9)
        if (u + 1) % N == 0:
            resid = sp.compute_residual_normsq(lr.sigma_dev, lr.U_dev)
            ref = c["resid"][u // N]
            np.testing.assert_allclose(resid, ref, rtol=1e-9)
            fit, fit_ref = 1 - np.sqrt(resid / c["normsq"]), 1 - np.sqrt(ref / c["normsq"])
            assert abs(fit - fit_ref) <= 1e-6 * abs(fit_ref)


def test_gpu_als_fp32_sampling_tracks_fp64(ftl):
    c = load_als(als_cases()[0])
    _, lr64, sp64, als64 = _setup(ftl, c, "fp64")
    _, lr32, sp32, als32 = _setup(ftl, c, "fp32")
    for upd in c["updates"]:
        als64.execute_ds_als_update(upd["j"], True, True, draws=upd["draws"])
        als32.execute_ds_als_update(upd["j"], True, True, draws=upd["draws"])
    r64 = sp64.compute_residual_normsq(lr64.sigma_dev, lr64.U_dev)
    r32 = sp32.compute_residual_normsq(lr32.sigma_dev, lr32.U_dev)
    assert abs(r32 - r64) <= 1e-3 * r64


def test_gpu_exact_als_update_matches_oracle(ftl):
    c = load_als(als_cases()[0])
    U, lr, sp, als = _setup(ftl, c)
    Uo = [u.copy() for u in c["U0"]]
    R = c["R"]
    for j in range(c["N"]):
        als.execute_exact_als_update(j, True, True)
        # numpy restatement of execute_exact_als_update (cpp_ext/als.hpp:222-270)
        G = np.ones((R, R))
        for k in range(c["N"]):
            if k != j:
                G = G * (Uo[k].T @ Uo[k])
        pinv = O.pinv_square(G, R, 1e-11)
        mt = np.zeros_like(Uo[j])
        part = c["vals"][:, None] * np.ones((1, R))
        for k in range(c["N"]):
            if k != j:
                part = part * Uo[k][c["idx"][:, k]]
        np.add.at(mt, c["idx"][:, j], part)
        Uj = mt @ pinv
        norms = np.sqrt((Uj ** 2).sum(axis=0))
        norms[norms <= 1e-7] = 1.0
        Uo[j] = Uj / norms
        np.testing.assert_allclose(U[j], Uo[j], rtol=0, atol=1e-9 * np.abs(Uo[j]).max())
        np.testing.assert_allclose(lr.sigma, norms, rtol=1e-9)


def test_gpu_downsampled_mttkrp_and_norms(ftl):
    c = load_als(als_cases()[1])
    rng = np.random.default_rng(3)
    sp = ftl.SparseTensor(c["idx"], c["vals"], "sort", dims=c["dims"])
    N, R, J = c["N"], 7, 500
    j = 2
    samples = np.stack([rng.integers(0, d, size=J) for d in c["dims"]], axis=1).astype(np.uint64)
    samples[: J // 2] = np.asarray(c["idx"][: J // 2], dtype=np.uint64)  # hit real fibers
    lhs = rng.normal(size=(J, R))
    out = np.zeros((c["dims"][j], R))
    sp.execute_downsampled_mttkrp_py(samples, lhs, j, out)
    keys = O.fiber_keys(c["idx"].astype(np.int64), c["dims"], j)
    skeys = O.fiber_keys(samples.astype(np.int64), c["dims"], j)
    ref = np.zeros_like(out)
    for i in range(J):
        for z in np.nonzero(keys == skeys[i])[0]:
            ref[c["idx"][z, j]] += c["vals"][z] * lhs[i]
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12)
    # LowRankTensor: renormalize every factor, sigma = product of norms
    U = [rng.normal(size=(d, R)) for d in c["dims"]]
    U0 = [u.copy() for u in U]
    lr = ftl.LowRankTensor(R, U)
    lr.renormalize_columns(-1)
    prod = np.ones(R)
    for k in range(N):
        nk = np.sqrt((U0[k] ** 2).sum(axis=0))
        prod *= nk
        np.testing.assert_allclose(U[k], U0[k] / nk, rtol=1e-13)
    np.testing.assert_allclose(lr.sigma, prod, rtol=1e-13)
    G = np.outer(prod, prod)
    for k in range(N):
        G = G * (U[k].T @ U[k])
    np.testing.assert_allclose(lr.get_normsq(), G.sum(), rtol=1e-11)


def test_gpu_als_fp32_rank64_four_modes_stays_finite(ftl):
    """Mixed-precision CP-ALS at R = 64 on a 4-mode Zipf tensor whose mode
    sizes (~4e4) far exceed what J = 1917 samples touch, so most factor rows
    become exact zeros after the first updates: factors, sigma and fit stay
    finite through a full eager sweep and a graph-captured one."""
    from fast_tensor_leverage_gb300.synthetic import sparse_powerlaw_tensor
    dims = [42030, 38493, 39731, 45257]
    idx, vals = sparse_powerlaw_tensor(dims, 142532, 1.1, seed=3, device="cuda")
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    rng = np.random.default_rng(4)
    lr = ftl.LowRankTensor(64, [rng.normal(size=(d, 64)) for d in dims], sync_host=False)
    lr.renormalize_columns(-1)
    als = ftl.ALS(lr, sp)
    als.initialize_ds_als(1917, "efficient", precision="fp32", seed=6)
    for j in range(4):
        als.execute_ds_als_update(j, True, True)
    als.capture_sweep()
    als.replay_sweep()
    torch.cuda.synchronize()
    for u in lr.U_dev:
        assert bool(torch.isfinite(u).all())
    assert bool(torch.isfinite(lr.sigma_dev).all())
    resid = sp.compute_residual_normsq(lr.sigma_dev, lr.U_dev)
    assert np.isfinite(resid)


def test_replay_after_eager_update_draws_fresh_uniforms(ftl):
    """An eager sampled update between two replays of a captured sweep
    advances the Philox stream the next replay draws from: the replay's last
    mode uses the uniforms at host counter + (N-1) 2NJ, none that the eager
    update already used."""
    from fast_tensor_leverage_gb300 import _lib
    from fast_tensor_leverage_gb300.synthetic import sparse_powerlaw_tensor
    dims, J, R = [3000, 2500, 2000], 512, 8
    N = len(dims)
    idx, vals = sparse_powerlaw_tensor(dims, 40000, 1.1, seed=5, device="cuda")
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    rng = np.random.default_rng(8)
    lr = ftl.LowRankTensor(R, [rng.normal(size=(d, R)) for d in dims], sync_host=False)
    lr.renormalize_columns(-1)
    als = ftl.ALS(lr, sp)
    als.initialize_ds_als(J, "efficient", precision="fp64", seed=6)
    for j in range(N):
        als.execute_ds_als_update(j, True, True)
    als.capture_sweep()
    als.replay_sweep()
    als.execute_ds_als_update(0, True, True)
    c = als.sampler.counter
    als.replay_sweep()
    torch.cuda.synchronize()
    expect = torch.empty(2 * N * J, dtype=torch.float64, device="cuda")
    _lib.call("ftl_philox_uniforms", expect.data_ptr(), 2 * N * J, als.sampler.seed, c + (N - 1) * 2 * N * J,
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(als._gdraws.reshape(-1), expect)
    assert als.sampler.counter == c + N * 2 * N * J


def test_gpu_exact_als_update_rank128_matches_numpy(ftl):
    """Exact update at the largest rank (R = 128: the solve stages 64 rows
    per block, the pseudo-inverse keeps its eigenvectors in global scratch)
    against the numpy restatement used above."""
    rng = np.random.default_rng(9)
    dims, nnz, R = [300, 200, 250], 6000, 128
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = rng.normal(size=nnz)
    U = [rng.normal(size=(d, R)) for d in dims]
    Uo = [u.copy() for u in U]
    lr = ftl.LowRankTensor(R, U)
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    als = ftl.ALS(lr, sp)
    als.initialize_ds_als(64, "efficient", precision="fp64", seed=1)
    j = 1
    als.execute_exact_als_update(j, True, True)
    G = np.ones((R, R))
    for k in range(3):
        if k != j:
            G = G * (Uo[k].T @ Uo[k])
    pinv = O.pinv_square(G, R, 1e-11)
    mt = np.zeros_like(Uo[j])
    part = vals[:, None] * np.ones((1, R))
    for k in range(3):
        if k != j:
            part = part * Uo[k][idx[:, k]]
    np.add.at(mt, idx[:, j], part)
    Uj = mt @ pinv
    norms = np.sqrt((Uj ** 2).sum(axis=0))
    norms[norms <= 1e-7] = 1.0
    np.testing.assert_allclose(U[j], Uj / norms, rtol=0, atol=1e-8 * np.abs(Uj / norms).max())
    np.testing.assert_allclose(lr.sigma, norms, rtol=1e-8)


def test_gpu_rrf_matches_oracle_and_is_gaussian(ftl):
    """SparseTensor.execute_rrf: the range finder of every mode against the
    oracle restatement with the same counter-based Gaussian vectors (FP32
    Box-Muller on the GPU vs FP64 in the oracle: 1e-5 of the largest entry),
    then unit columns and sigma = product of the column norms."""
    c = load_als(als_cases()[1])
    R, seed = 9, 77
    rows = [d + 3 for d in c["dims"]]          # factors may have more rows than the tensor
    U = [np.zeros((r, R)) for r in rows]
    lr = ftl.LowRankTensor(R, U)
    sp = ftl.SparseTensor(c["idx"], c["vals"], "sort", dims=c["dims"])
    sp.execute_rrf(lr, seed=seed)
    Uo = O.rrf(c["idx"], c["vals"], c["dims"], rows, R, seed)
    sig = np.ones(R)
    for k in range(c["N"]):
        n = np.linalg.norm(Uo[k], axis=0)
        n[n <= 1e-7] = 1.0
        sig *= n
        np.testing.assert_allclose(U[k], Uo[k] / n, rtol=0, atol=1e-5)
        assert np.all(U[k][c["dims"][k]:] == 0.0)
    np.testing.assert_allclose(lr.sigma, sig, rtol=1e-5)
    # one nonzero of value 1 per row, all in distinct fibers: rows = the vectors
    n_rows, R2 = 20000, 64
    idx = np.stack([np.arange(n_rows), np.arange(n_rows) % 97, np.arange(n_rows) // 97], axis=1).astype(np.uint32)
    sp2 = ftl.SparseTensor(idx, np.ones(n_rows), "sort", dims=[n_rows, 97, n_rows // 97 + 1])
    out = torch.empty((n_rows, R2), dtype=torch.float64, device="cuda")
    from fast_tensor_leverage_gb300 import _lib
    rrows, rkeys, rvals = sp2.rows[0]
    _lib.call("ftl_sparse_rrf", rrows.data_ptr(), rkeys.data_ptr(), rvals.data_ptr(), sp2.nnz, R2, 5, 0,
              out.data_ptr(), n_rows, torch.cuda.current_stream().cuda_stream)
    g = out.cpu().numpy()
    assert abs(g.mean()) < 0.005 and abs(g.var() - 1.0) < 0.01
    assert abs(((g - g.mean()) ** 4).mean() / g.var() ** 2 - 3.0) < 0.05
    corr = np.corrcoef(g[:, :8].T)
    assert np.abs(corr - np.eye(8)).max() < 0.05
    ref = np.stack([O.fiber_normals(5, 0, int(k), R2) for k in rkeys[:50].cpu().numpy()])
    np.testing.assert_allclose(g[rrows[:50].cpu().numpy()], ref, rtol=0, atol=1e-5)


from tests._golden import bb_cases, load_bb  # noqa: E402


def _bb_rhs(ftl, c, f32=False):
    if c["kind"] == "lowrank":
        V = [v.copy() for v in c["V"]]
        t = ftl.LowRankTensor(c["Rr"], 10000, V)
        t.set_sigma(c["sv"])
        return t
    return ftl.DenseTensor(c["T"].astype(np.float32) if f32 else c["T"], 10000)


@pytest.mark.parametrize("name", bb_cases())
def test_gpu_blackbox_als_matches_reference_golden(ftl, name):
    """CP-ALS against a low-rank / dense right-hand side (black_box_tensor.hpp:
    21-67) vs the reference with the same uniforms: samples identical,
    factors within 1e-9 of the largest entry, sigma 1e-9 relative, and for
    the low-rank case the residual 1e-9 and the fit 1e-6 relative."""
    c = load_bb(name)
    rhs = _bb_rhs(ftl, c)
    U = [u.copy() for u in c["U0"]]
    lr = ftl.LowRankTensor(c["R"], U)
    lr.set_sigma(c["sigma0"])
    als = ftl.ALS(lr, rhs)
    als.initialize_ds_als(c["J"], "efficient", precision="fp64")
    N = c["N"]
    for u, upd in enumerate(c["updates"]):
        j = upd["j"]
        als.execute_ds_als_update(j, True, True, draws=upd["draws"])
        samples = als.sampler.samples_dev.cpu().numpy().view(np.uint64)
        rows = [k for k in range(N) if k != j]
        assert np.array_equal(samples[rows], upd["samples"][rows]), f"update {u}"
        np.testing.assert_allclose(U[j], upd["U"], rtol=0, atol=1e-9 * np.abs(upd["U"]).max())
        np.testing.assert_allclose(lr.sigma, upd["sigma"], rtol=1e-9)
        if c["kind"] == "lowrank" and (u + 1) % N == 0:
            resid, ref = rhs.compute_residual_normsq(lr.sigma, U), float(c[f"resid_{u // N}"])
            np.testing.assert_allclose(resid, ref, rtol=1e-9)
            nrm = float(c["normsq_rhs"])
            fit, fit_ref = 1 - np.sqrt(resid / nrm), 1 - np.sqrt(ref / nrm)
            assert abs(fit - fit_ref) <= 1e-6 * abs(fit_ref)
    if c["kind"] == "lowrank":
        S = c["mat_S"]
        for jj in (1, N):
            m = np.zeros_like(c[f"mat_{jj}"])
            rhs.materialize_rhs(S, jj, m)
            np.testing.assert_allclose(m, c[f"mat_{jj}"], rtol=1e-12, atol=1e-12)
        ev = np.zeros(S.shape[0])
        rhs.evaluate_indices(S.astype(np.uint32), ev)
        np.testing.assert_allclose(ev, c["eval"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(rhs.get_normsq(), float(c["normsq_rhs"]), rtol=1e-12)


@pytest.mark.parametrize("name", bb_cases())
def test_gpu_blackbox_downsampled_mttkrp_and_exact_update(ftl, name):
    """Tensor-API MTTKRP (execute_downsampled_mttkrp_py) vs explicit fibers,
    the FP32 dense tensor vs FP64, the dense residual, and (low-rank) the
    exact ALS update vs its numpy statement (low_rank_tensor.hpp:147-180)."""
    c = load_bb(name)
    rng = np.random.default_rng(2)
    rhs = _bb_rhs(ftl, c)
    o = O.OracleLowRankRHS(c["V"], c["sv"]) if c["kind"] == "lowrank" else O.OracleDenseRHS(c["T"])
    J, R, j = 700, 7, 1
    S = np.stack([rng.integers(0, d, size=J) for d in c["dims"]], axis=1).astype(np.uint64)
    L = rng.normal(size=(J, R))
    out = np.zeros((c["dims"][j], R))
    rhs.execute_downsampled_mttkrp_py(S, L, j, out)
    want = o.fibers(S.astype(np.int64), j).T @ L
    np.testing.assert_allclose(out, want, rtol=0, atol=1e-11 * np.abs(want).max())
    if c["kind"] == "dense":
        r32 = _bb_rhs(ftl, c, f32=True)
        o32 = np.zeros_like(out)
        r32.execute_downsampled_mttkrp_py(S, L, j, o32)
        np.testing.assert_allclose(o32, want, rtol=0, atol=1e-5 * np.abs(want).max())
        Ul = [rng.normal(size=(d, 3)) for d in c["dims"]]
        sg = rng.random(3) + 0.5
        model = np.einsum("r,ir,jr,kr->ijk", sg, *Ul)
        np.testing.assert_allclose(rhs.compute_residual_normsq(sg, Ul), ((c["T"] - model) ** 2).sum(), rtol=1e-11)
        np.testing.assert_allclose(rhs.get_normsq(), (c["T"] ** 2).sum(), rtol=1e-12)
        return
    Rl = 5
    U = [rng.normal(size=(d, Rl)) for d in c["dims"]]
    Uo = [u.copy() for u in U]
    lr = ftl.LowRankTensor(Rl, U)
    als = ftl.ALS(lr, rhs)
    als.execute_exact_als_update(j, True, False)
    G = np.ones((Rl, Rl))
    M = np.outer(c["sv"], np.ones(Rl))
    for k in range(c["N"]):
        if k != j:
            G = G * (Uo[k].T @ Uo[k])
            M = M * (c["V"][k].T @ Uo[k])
    mt = c["V"][j] @ M
    Uj = mt @ O.pinv_square(G, Rl, 1e-11)
    n = np.linalg.norm(Uj, axis=0)
    np.testing.assert_allclose(U[j], Uj / n, rtol=0, atol=1e-9 * np.abs(Uj / n).max())


def _pinv_gpu(M, R, target, cap=None):
    from fast_tensor_leverage_gb300 import _lib
    Md = torch.as_tensor(M, device="cuda")
    out = torch.empty_like(Md)
    vs = torch.empty_like(Md)
    capd = None if cap is None else torch.tensor([cap], dtype=torch.int64, device="cuda")
    _lib.call("ftl_pinv_square", Md.data_ptr(), R, target, None if capd is None else capd.data_ptr(), 1e-11,
              out.data_ptr(), vs.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


def _spd(rng, R, lam):
    Q, _ = np.linalg.qr(rng.normal(size=(R, R)))
    return (Q * lam) @ Q.T


@pytest.mark.parametrize("R", [1, 5, 25, 64, 128])
def test_pinv_square_well_conditioned(ftl, R):
    """Positive definite Grams (the Cholesky path): the pseudo-inverse equals
    the oracle's eigen-based one to 1e-11 relative (Frobenius)."""
    rng = np.random.default_rng(90 + R)
    B = rng.normal(size=(3 * R, R))
    M = B.T @ B * 1e3
    ref = O.pinv_square(M, R, 1e-11)
    got = _pinv_gpu(M, R, R)
    assert np.linalg.norm(got - ref) <= 1e-11 * np.linalg.norm(ref)


@pytest.mark.parametrize("R", [6, 25, 100])
def test_pinv_square_drops_eigenvalues_like_the_reference(ftl, R):
    """Eigenvalues at or below the 1e-11 cut, exact zeros (rank-deficient
    Grams) and a rank cap below R take the eigen path: the same eigenpairs are
    kept as in the oracle."""
    rng = np.random.default_rng(190 + R)
    lam = np.exp(rng.uniform(-2, 2, size=R))
    # an eigenvalue below the cut: dropped
    lam1 = lam.copy()
    lam1[0] = 4e-12
    M = _spd(rng, R, lam1)
    ref = O.pinv_square(M, R, 1e-11)
    got = _pinv_gpu(M, R, R)
    assert np.linalg.norm(got - ref) <= 1e-8 * np.linalg.norm(ref)
    # rank-deficient Gram (three exact zero directions)
    B = rng.normal(size=(R, R - 3))
    M = B @ B.T
    ref = O.pinv_square(M, R, 1e-11)
    got = _pinv_gpu(M, R, R)
    assert np.linalg.norm(got - ref) <= 1e-8 * np.linalg.norm(ref)
    # rank cap below R (fewer unique samples than R): the R - cap smallest dropped
    M = _spd(rng, R, lam)
    for cap in (R - 2, 1):
        ref = O.pinv_square(M, cap, 1e-11)
        assert np.linalg.norm(_pinv_gpu(M, R, R, cap=cap) - ref) <= 1e-9 * np.linalg.norm(ref)
        assert np.linalg.norm(_pinv_gpu(M, R, cap) - ref) <= 1e-9 * np.linalg.norm(ref)


@pytest.mark.parametrize("R,j", [(25, 0), (48, 1), (100, 2)])
def test_sparse_mttkrp_rows_against_numpy(ftl, R, j):
    """The row-grouped sparse MTTKRP against numpy, 1e-13 relative to the
    largest entry: queries are the fibers of a random set of nonzeros plus
    absent fibers, with repeats."""
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(300 + R)
    dims = [70, 50, 40]
    nnz = 20000
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = rng.lognormal(0.0, 1.0, size=nnz)
    sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
    st = torch.cuda.current_stream().cuda_stream
    J = 3000
    keys_all = O.fiber_keys(idx, dims, j)
    q = np.concatenate([keys_all[rng.integers(0, nnz, size=J - 200)],
                        rng.integers(0, 2**40, size=200).astype(np.uint64)])
    keys = torch.from_numpy(q.view(np.int64)).cuda()
    nb = _lib.ws_bytes("dedup", J)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    ukeys = torch.empty(J, dtype=torch.int64, device="cuda")
    urep = torch.empty(J, dtype=torch.int32, device="cuda")
    ucnt = torch.empty(J, dtype=torch.int32, device="cuda")
    nu = torch.zeros(1, dtype=torch.int64, device="cuda")
    _lib.call("ftl_dedup", keys.data_ptr(), J, ws.data_ptr(), nb, ukeys.data_ptr(), urep.data_ptr(),
              ucnt.data_ptr(), nu.data_ptr(), st)
    h = torch.from_numpy(rng.normal(size=(J, R))).cuda()
    w = torch.from_numpy(rng.uniform(0.5, 2.0, size=J)).cuda()
    rrows, rkeys, rvals = sp.rows[j]
    mb = _lib.ws_bytes("mttkrp_rows", J, R)
    mws = torch.empty(mb, dtype=torch.uint8, device="cuda")
    out = torch.empty((dims[j], R), dtype=torch.float64, device="cuda")
    _lib.call("ftl_sparse_mttkrp_rows", rrows.data_ptr(), rkeys.data_ptr(), rvals.data_ptr(), sp.nnz,
              ukeys.data_ptr(), urep.data_ptr(), ucnt.data_ptr(), nu.data_ptr(), J, J, w.data_ptr(),
              h.data_ptr(), R, mws.data_ptr(), mb, out.data_ptr(), dims[j], st)
    got = out.cpu().numpy()
    n = int(nu.item())
    uk, ur, uc = ukeys.cpu().numpy()[:n].view(np.uint64), urep.cpu().numpy()[:n], ucnt.cpu().numpy()[:n]
    hh, ww = h.cpu().numpy(), w.cpu().numpy()
    pos = {int(k): u for u, k in enumerate(uk)}
    ref = np.zeros((dims[j], R))
    for z in range(nnz):
        u = pos.get(int(keys_all[z]))
        if u is not None:
            ref[idx[z, j]] += vals[z] * ww[ur[u]] * uc[u] * hh[ur[u]]
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() <= 1e-13 * scale


@pytest.mark.parametrize("name", als_cases())
def test_als_handle_matches_reference_golden(ftl, name):
    """The native handle path (ftl_sparse_create, ftl_als_create, set_factor,
    set_sigma, ftl_als_update with injected uniforms, ftl_als_fit) against the
    reference's recorded ALS: the tolerances of the Python-path test."""
    import ctypes
    from fast_tensor_leverage_gb300 import _lib
    c = load_als(name)
    N, R, J = c["N"], c["R"], c["J"]
    st = torch.cuda.current_stream().cuda_stream
    idx = np.ascontiguousarray(c["idx"], dtype=np.uint32)
    vals = np.ascontiguousarray(c["vals"], dtype=np.float64)
    dims = (ctypes.c_int64 * N)(*c["dims"])
    X, A = ctypes.c_void_p(), ctypes.c_void_p()
    _lib.call("ftl_sparse_create", idx.ctypes.data, vals.ctypes.data, idx.shape[0], N, dims, 1, st, ctypes.byref(X))
    try:
        nsq = ctypes.c_double()
        _lib.call("ftl_sparse_normsq", X, ctypes.byref(nsq))
        assert abs(nsq.value - c["normsq"]) <= 1e-12 * c["normsq"]
        _lib.call("ftl_als_create", X, R, J, 0, 1, ctypes.byref(A))
        for k in range(N):
            u0 = np.ascontiguousarray(c["U0"][k])
            _lib.call("ftl_als_set_factor", A, k, u0.ctypes.data, 1, st)
        s0 = np.ascontiguousarray(c["sigma0"])
        _lib.call("ftl_als_set_sigma", A, s0.ctypes.data, 1, st)

        def dev_view(ptr, shape, typestr):
            v = type("V", (), {"__cuda_array_interface__": {
                "shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3}})()
            return torch.as_tensor(v, device="cuda")

        sp_ptr, sg_ptr = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.call("ftl_als_samples", A, ctypes.byref(sp_ptr))
        _lib.call("ftl_als_sigma", A, ctypes.byref(sg_ptr))
        samples_t = dev_view(sp_ptr.value, (N, J), "<i8")
        sigma_t = dev_view(sg_ptr.value, (R,), "<f8")
        for u, upd in enumerate(c["updates"]):
            j = upd["j"]
            dr = torch.from_numpy(upd["draws"]).cuda()
            _lib.call("ftl_als_update", A, j, 1, 1, dr.data_ptr(), st)
            torch.cuda.synchronize()
            samples = samples_t.cpu().numpy().view(np.uint64)
            rows = [k for k in range(N) if k != j]
            assert np.array_equal(samples[rows], upd["samples"][rows]), f"update {u}: samples differ"
            up = ctypes.c_void_p()
            _lib.call("ftl_als_factor", A, j, ctypes.byref(up))
            Uj = dev_view(up.value, (c["dims"][j], R), "<f8").cpu().numpy()
            np.testing.assert_allclose(Uj, upd["U"], rtol=0, atol=1e-9 * np.abs(upd["U"]).max())
            np.testing.assert_allclose(sigma_t.cpu().numpy(), upd["sigma"], rtol=1e-9)
            if (u + 1) % N == 0:
                fit, resid = ctypes.c_double(), ctypes.c_double()
                _lib.call("ftl_als_fit", A, ctypes.byref(fit), ctypes.byref(resid), st)
                ref = c["resid"][u // N]
                np.testing.assert_allclose(resid.value, ref, rtol=1e-9)
                fit_ref = 1 - np.sqrt(ref / c["normsq"])
                assert abs(fit.value - fit_ref) <= 1e-6 * abs(fit_ref)
    finally:
        _lib.call("ftl_als_destroy", A)
        _lib.call("ftl_sparse_destroy", X)


def test_als_handle_rrf_mixed_precision_runs(ftl):
    """Range-finder initialisation and Philox-driven mixed-precision updates
    through the handle: the fit is finite and the sweep improves on the
    initial model."""
    import ctypes
    from fast_tensor_leverage_gb300 import _lib
    rng = np.random.default_rng(123)
    dims = [300, 200, 100]
    nnz = 30000
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.ascontiguousarray(np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32))
    vals = np.log1p(rng.lognormal(size=nnz))
    st = torch.cuda.current_stream().cuda_stream
    X, A = ctypes.c_void_p(), ctypes.c_void_p()
    _lib.call("ftl_sparse_create", idx.ctypes.data, vals.ctypes.data, nnz, 3, (ctypes.c_int64 * 3)(*dims), 1, st,
              ctypes.byref(X))
    try:
        _lib.call("ftl_als_create", X, 10, 4096, 1, 99, ctypes.byref(A))
        _lib.call("ftl_als_init_rrf", A, 5, st)
        f0 = ctypes.c_double()
        _lib.call("ftl_als_fit", A, ctypes.byref(f0), None, st)
        for _ in range(3):
            for j in range(3):
                _lib.call("ftl_als_update", A, j, 1, 1, None, st)
        f1 = ctypes.c_double()
        _lib.call("ftl_als_fit", A, ctypes.byref(f1), None, st)
        assert np.isfinite(f1.value) and f1.value > f0.value
    finally:
        _lib.call("ftl_als_destroy", A)
        _lib.call("ftl_sparse_destroy", X)


def test_multiply_random_factor_entries(ftl):
    """LowRankTensor.multiply_random_factor_entries(rho, A): each entry
    scaled by A with probability rho (low_rank_tensor.hpp:289-303), host
    arrays mirrored, reproducible with a seed."""
    rng = np.random.default_rng(8)
    U = [rng.normal(size=(5000, 8)) for _ in range(3)]
    orig = [u.copy() for u in U]
    lr = ftl.LowRankTensor(8, U)
    lr.multiply_random_factor_entries(0.01, 10.0, seed=3)
    changed = 0
    for u, o in zip(U, orig):
        hit = u != o
        np.testing.assert_array_equal(u[hit], o[hit] * 10.0)
        changed += int(hit.sum())
    frac = changed / (3 * 5000 * 8)
    assert 0.008 < frac < 0.012, frac
    U2 = [o.copy() for o in orig]
    lr2 = ftl.LowRankTensor(8, U2)
    lr2.multiply_random_factor_entries(0.01, 10.0, seed=3)
    for a, b in zip(U, U2):
        np.testing.assert_array_equal(a, b)
