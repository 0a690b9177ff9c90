"""GPU: continuous-batching serving loop.  Every request's result in the mix
equals the same request run alone: sampling bit-exactly (same seed, the
packed launch runs the per-sample code of the single launch), CP-ALS up to
the order of floating-point atomic additions in the MTTKRP (factors within
1e-9 of the largest entry, fit within 1e-9).  The HBM budget is never
exceeded and concurrent sampling requests share packed launches."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ftl():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fast_tensor_leverage_gb300 as m
    return m


def _sparse(rng, dims, nnz):
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    return idx, np.log1p(rng.lognormal(0.0, 1.0, size=nnz))


def _requests(S):
    rng = np.random.default_rng(12)
    reqs = []
    specs = [(3, 2000, 16, 3000, 4, "fp32"), (4, 900, 16, 5000, 1, "fp32"), (3, 40000, 32, 8000, 9, "fp32"),
             (5, 300, 8, 2000, 0, "fp64"), (3, 7000, 16, 1000, 2, "fp32"), (6, 120, 8, 4000, 9, "fp32")]
    for n, (N, I, R, J, j, prec) in enumerate(specs):
        factors = [rng.normal(size=(I + 37 * k, R)) for k in range(N)]
        reqs.append(S.SampleRequest(factors, J, j, prec, seed=100 + n))
    for n, (dims, nnz, R, J) in enumerate([([40, 30, 20], 2000, 8, 400), ([25, 60, 35], 3000, 6, 300)]):
        idx, vals = _sparse(rng, dims, nnz)
        reqs.append(S.ALSRequest(idx, vals, dims, R, J, sweeps=3, precision="fp64", seed=5 + n,
                                 sampler_seed=9 + n))
    return reqs


def test_mix_equals_alone(ftl):
    from fast_tensor_leverage_gb300 import serving as S
    reqs = _requests(S)
    sizes = [S.estimate_bytes(r) for r in reqs]
    budget = sum(sorted(sizes)[-3:])  # forces some requests to wait
    eng = S.ServingEngine(budget, max_active=8)
    # a burst of three requests (two share R = 16 and pack into one launch),
    # then the rest spread out while those are on the device
    arrivals = [(0.0 if i < 3 else 0.002 * i, r) for i, r in enumerate(reqs)]
    done = eng.run(arrivals)
    assert len(done) == len(reqs)
    assert eng.max_in_use <= budget
    by_id = {h.rid: h for h in done}
    for rid, r in enumerate(reqs):
        res = by_id[rid].result
        if isinstance(r, S.SampleRequest):
            s = ftl.Sampler(r.factors, r.J, r.factors[0].shape[1], "efficient", precision=r.precision, seed=r.seed)
            samples, h, w = s.draw(r.j)
            N = len(r.factors)
            rows = [k for k in range(N) if k != r.j]
            assert np.array_equal(res["samples"][rows], samples.cpu().numpy().view(np.uint64)[rows])
            assert np.array_equal(res["h"], h.cpu().numpy())
            assert np.array_equal(res["weights"], w.cpu().numpy())
        else:
            U = S.GaussianFactors(r.dims, r.R, seed=r.seed).materialize(torch.device("cuda", 0))
            lr = ftl.LowRankTensor(r.R, U, sync_host=False)
            lr.renormalize_columns(-1)
            sp = ftl.SparseTensor(r.idx, r.vals, "sort", dims=r.dims)
            als = ftl.ALS(lr, sp)
            als.initialize_ds_als(r.J, "efficient", precision=r.precision, seed=r.sampler_seed)
            for _ in range(r.sweeps):
                for j in range(len(r.dims)):
                    als.execute_ds_als_update(j, True, True)
            for k in range(len(r.dims)):
                ref = lr.U_dev[k].cpu().numpy()
                np.testing.assert_allclose(res["U"][k], ref, rtol=0, atol=1e-9 * np.abs(ref).max())
            resid = sp.compute_residual_normsq(lr.sigma_dev, lr.U_dev)
            fit = 1.0 - np.sqrt(max(resid, 0.0) / sp.get_normsq())
            assert abs(res["fit"] - fit) <= 1e-9
    assert eng.packed_launches < sum(isinstance(r, S.SampleRequest) for r in reqs)
    lat = S.latency_stats(done)
    assert lat["count"] == len(reqs) and lat["p99_ms"] >= lat["p50_ms"] > 0


def test_captured_als_sweep_equals_eager(ftl):
    rng = np.random.default_rng(4)
    dims, R, J = [30, 45, 25], 7, 350
    flat = rng.choice(int(np.prod(dims)), size=2500, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = rng.random(2500) + 0.5
    out = []
    for graph in (False, True):
        r2 = np.random.default_rng(8)
        U = [r2.normal(size=(d, R)) for d in dims]
        lr = ftl.LowRankTensor(R, U, sync_host=False)
        lr.renormalize_columns(-1)
        sp = ftl.SparseTensor(idx, vals, "sort", dims=dims)
        als = ftl.ALS(lr, sp)
        als.initialize_ds_als(J, "efficient", precision="fp64", seed=21)
        for j in range(3):
            als.execute_ds_als_update(j, True, True)
        if graph:
            als.capture_sweep()
            for _ in range(3):
                als.replay_sweep()
        else:
            for _ in range(3):
                for j in range(3):
                    als.execute_ds_als_update(j, True, True)
        torch.cuda.synchronize()
        out.append([u.cpu().numpy() for u in lr.U_dev])
    for a, b in zip(*out):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-9 * np.abs(b).max())
