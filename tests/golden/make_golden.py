"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference C++ sampler (vbharadwaj-bk/fast_tensor_leverage,
cpp_ext/efficient_krp_sampler.hpp and cpp_ext/partition_tree.hpp), compiled
from its sources by `make -C oracle ref` into oracle/_ref/ftl_ref*.so, on
seeded inputs with injected uniforms, and stores inputs, uniforms and the
reference's outputs (sample indices, h, weights, node Grams).

    make -C oracle ref && python tests/golden/make_golden.py [--only bb]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "oracle" / "_ref"))

import ftl_ref  # noqa: E402

# name: (N, dims, R, J, j, seed, heavy_rows)
KRP_CASES = {
    "krp_readme_shape": (4, [1000] * 4, 8, 2000, 5, 11, 0.0),
    "krp_partial_leaf_excl1": (3, [1001, 1001, 1001], 8, 1500, 1, 12, 0.0),
    "krp_ragged_r25_excl0": (3, [300, 1500, 64], 25, 1000, 0, 13, 0.0),
    "krp_rows_lt_rank": (3, [20, 20, 20], 32, 800, 4, 14, 0.0),
    "krp_r32_heavy_excl_last": (3, [1024, 512, 700], 32, 800, 2, 15, 0.01),
}

# name: (n, F, R, J, seed)
TREE_CASES = {
    "tree_partial_n1001_f8": (1001, 8, 8, 1000, 21),
    "tree_complete_n1024_f32": (1024, 32, 32, 600, 22),
    "tree_f1_n13": (13, 1, 13, 500, 23),
}


def make_factors(rng, dims, R, heavy):
    U = []
    for n in dims:
        u = rng.normal(size=(n, R))
        if heavy > 0:
            rows = rng.choice(n, size=max(1, int(heavy * n)), replace=False)
            u[rows] *= 100.0
        U.append(u)
    return U


# name: (dims, nnz, R, J, sweeps, seed)
ALS_CASES = {
    "als_sparse_3mode_r8": ([40, 30, 20], 2000, 8, 400, 2, 31),
    "als_sparse_4mode_r5_ragged": ([17, 50, 9, 23], 1500, 5, 300, 2, 32),
}


def make_als_case(name, dims, nnz, R, J, sweeps, seed):
    """Reference ALS (cpp_ext/als.hpp via the harness's InjectedALS): factors
    renormalised once (renormalize_columns(-1), as the reference's benchmark
    does), then `sweeps` sweeps of execute_ds_als_update(j, True, True) with
    injected uniforms; records every update's samples and factor, and the
    residual after each sweep."""
    rng = np.random.default_rng(seed)
    N = len(dims)
    flat = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idx = np.stack(np.unravel_index(flat, dims), axis=1).astype(np.uint32)
    vals = np.log1p(rng.lognormal(0.0, 1.0, size=nnz))
    U = [rng.normal(size=(d, R)) for d in dims]
    lr = ftl_ref.LowRankTensor(R, U)
    lr.renormalize_columns(-1)
    sigma0 = np.zeros(R)
    lr.get_sigma(sigma0, -1)
    out = {f"U0_{k}": U[k].copy() for k in range(N)}
    sp = ftl_ref.SparseTensor(idx, vals, "sort")
    als = ftl_ref.InjectedALS(lr, sp)
    als.initialize_ds_als(J)
    upd = 0
    for sw in range(sweeps):
        for j in range(N):
            d = rng.random(2 * N * J)
            als.set_draws(d)
            als.execute_ds_als_update(j, True, True)
            smp = np.zeros((N, J), dtype=np.uint64)
            als.get_samples(smp)
            sg = np.zeros(R)
            lr.get_sigma(sg, -1)
            out[f"draws_{upd}"] = d
            out[f"samples_{upd}"] = smp
            out[f"U_{upd}"] = U[j].copy()
            out[f"sigma_{upd}"] = sg
            upd += 1
        sg = np.zeros(R)
        lr.get_sigma(sg, -1)
        out[f"resid_{sw}"] = np.array(sp.compute_residual_normsq(sg, U))
    out.update(dims=np.array(dims), idx=idx, vals=vals, sigma0=sigma0, R=R, J=J, sweeps=sweeps,
               normsq=np.array(sp.get_normsq()))
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "written")


# name: (kind, dims, rhs rank, R, J, sweeps, seed)
BB_CASES = {
    "bb_lowrank_4mode_r6": ("lowrank", [30, 22, 18, 25], 4, 6, 500, 2, 41),
    "bb_dense_3mode_r5": ("dense", [16, 13, 11], 3, 5, 400, 2, 42),
}


def make_blackbox_case(name, kind, dims, Rr, R, J, sweeps, seed):
    """Reference ALS against a black-box right-hand side (BlackBoxTensor::
    execute_downsampled_mttkrp, cpp_ext/black_box_tensor.hpp:21-67): a
    low-rank tensor (LowRankTensor(Rr, 10000, V)) or a dense one
    (DenseTensor<double>: rank-Rr tensor plus 10% Gaussian noise), injected
    uniforms, every update's samples and factor; for the low-rank case also
    the residual after each sweep and materialize_rhs / evaluate_indices
    vectors."""
    rng = np.random.default_rng(seed)
    N = len(dims)
    V = [rng.normal(size=(d, Rr)) for d in dims]
    out = {f"V_{k}": V[k] for k in range(N)}
    if kind == "lowrank":
        rhs = ftl_ref.LowRankTensor(Rr, 10000, V)
        sv = np.zeros(Rr)
        rhs.get_sigma(sv, -1)
        out["sv"] = sv
        out["normsq_rhs"] = np.array(rhs.get_normsq())
        S = np.stack([rng.integers(0, d, size=60) for d in dims], axis=1).astype(np.uint64)
        out["mat_S"] = S
        for jj in (1, N):
            m = np.zeros((60, dims[jj] if jj < N else Rr))
            rhs.materialize_rhs(S, jj, m)
            out[f"mat_{jj}"] = m
        ev = np.zeros(60)
        rhs.evaluate_indices(S.astype(np.uint32), ev)
        out["eval"] = ev
    else:
        T = np.einsum("ir,jr,kr->ijk", *V) + 0.1 * rng.normal(size=dims)
        T = np.ascontiguousarray(T)
        rhs = ftl_ref.DenseTensor(T, 10000)
        out["T"] = T
    U = [rng.normal(size=(d, R)) for d in dims]
    lr = ftl_ref.LowRankTensor(R, U)
    lr.renormalize_columns(-1)
    sigma0 = np.zeros(R)
    lr.get_sigma(sigma0, -1)
    out.update({f"U0_{k}": U[k].copy() for k in range(N)})
    als = ftl_ref.InjectedALS(lr, rhs)
    als.initialize_ds_als(J)
    upd = 0
    for sw in range(sweeps):
        for j in range(N):
            d = rng.random(2 * N * J)
            als.set_draws(d)
            als.execute_ds_als_update(j, True, True)
            smp = np.zeros((N, J), dtype=np.uint64)
            als.get_samples(smp)
            sg = np.zeros(R)
            lr.get_sigma(sg, -1)
            out[f"draws_{upd}"] = d
            out[f"samples_{upd}"] = smp
            out[f"U_{upd}"] = U[j].copy()
            out[f"sigma_{upd}"] = sg
            upd += 1
        if kind == "lowrank":
            sg = np.zeros(R)
            lr.get_sigma(sg, -1)
            out[f"resid_{sw}"] = np.array(rhs.compute_residual_normsq(sg, U))
    out.update(kind=kind, dims=np.array(dims), Rr=Rr, R=R, J=J, sweeps=sweeps, sigma0=sigma0)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "written")


def main() -> None:
    if "--only" in sys.argv:
        which = sys.argv[sys.argv.index("--only") + 1]
        if which == "bb":
            for name, args in BB_CASES.items():
                make_blackbox_case(name, *args)
            return
        raise SystemExit(f"unknown --only {which}")
    for name, (N, dims, R, J, j, seed, heavy) in KRP_CASES.items():
        rng = np.random.default_rng(seed)
        U = make_factors(rng, dims, R, heavy)
        draws = rng.random(2 * N * J)
        s = ftl_ref.RefSampler(U, J, R)
        samples = np.zeros((N, J), dtype=np.uint64)
        s.draw(j, samples, draws)
        h = np.zeros((J, R))
        w = np.zeros(J)
        s.get_h(h)
        s.get_weights(w)
        out = {f"U{k}": U[k] for k in range(N)}
        out.update(N=N, R=R, J=J, j=j, draws=draws, samples=samples, h=h, weights=w)
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, "written")
    for name, args in ALS_CASES.items():
        make_als_case(name, *args)
    for name, args in BB_CASES.items():
        make_blackbox_case(name, *args)
    for name, (n, F, R, J, seed) in TREE_CASES.items():
        rng = np.random.default_rng(seed)
        U = rng.normal(size=(n, R))
        scaled_h = rng.normal(size=(J, R))
        h = rng.normal(size=(J, R))
        draws = rng.random(J)
        t = ftl_ref.RefPartitionTree(n, F, J, R)
        t.build_tree(U)
        geom = t.geometry()
        G = np.zeros((geom["node_count"], R, R))
        t.get_G(G)
        h_out = h.copy()
        samples = np.zeros(J, dtype=np.uint64)
        t.PTSample(U, h_out, scaled_h, samples, draws)
        iu = np.triu_indices(R)
        np.savez_compressed(
            HERE / f"{name}.npz", n=n, F=F, R=R, J=J, U=U, h=h, scaled_h=scaled_h, draws=draws,
            G_packed=G[:, iu[0], iu[1]], samples=samples, h_out=h_out,
            geometry=np.array([geom[k] for k in (
                "leaf_count", "node_count", "lfill_level", "lfill_count", "total_levels",
                "nodes_upto_lfill", "nodes_before_lfill", "complete_level_offset")], dtype=np.int64))
        print(name, "written")


if __name__ == "__main__":
    main()
