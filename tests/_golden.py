"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def krp_cases():
    return sorted(p.stem for p in GOLDEN.glob("krp_*.npz"))


def tree_cases():
    return sorted(p.stem for p in GOLDEN.glob("tree_*.npz"))


def load_krp(name):
    z = np.load(GOLDEN / f"{name}.npz")
    N = int(z["N"])
    return dict(
        U=[z[f"U{k}"] for k in range(N)], N=N, R=int(z["R"]), J=int(z["J"]), j=int(z["j"]),
        draws=z["draws"], samples=z["samples"], h=z["h"], weights=z["weights"])


def load_tree(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return {k: z[k] for k in z.files}


def included_rows(N, j):
    return [k for k in range(N) if k != j]


def als_cases():
    return sorted(p.stem for p in GOLDEN.glob("als_*.npz"))


def load_als(name):
    z = np.load(GOLDEN / f"{name}.npz")
    dims = [int(d) for d in z["dims"]]
    N = len(dims)
    c = dict(dims=dims, N=N, R=int(z["R"]), J=int(z["J"]), sweeps=int(z["sweeps"]), idx=z["idx"],
             vals=z["vals"], sigma0=z["sigma0"], normsq=float(z["normsq"]),
             U0=[z[f"U0_{k}"] for k in range(N)])
    n_upd = c["sweeps"] * N
    c["updates"] = [dict(j=u % N, draws=z[f"draws_{u}"], samples=z[f"samples_{u}"], U=z[f"U_{u}"],
                         sigma=z[f"sigma_{u}"]) for u in range(n_upd)]
    c["resid"] = [float(z[f"resid_{s}"]) for s in range(c["sweeps"])]
    return c


def bb_cases():
    return sorted(p.stem for p in GOLDEN.glob("bb_*.npz"))


def load_bb(name):
    z = np.load(GOLDEN / f"{name}.npz")
    dims = [int(d) for d in z["dims"]]
    N = len(dims)
    c = {k: z[k] for k in z.files}
    c.update(kind=str(z["kind"]), dims=dims, N=N, R=int(z["R"]), Rr=int(z["Rr"]), J=int(z["J"]),
             sweeps=int(z["sweeps"]), V=[z[f"V_{k}"] for k in range(N)], U0=[z[f"U0_{k}"] for k in range(N)])
    c["updates"] = [dict(j=u % N, draws=z[f"draws_{u}"], samples=z[f"samples_{u}"], U=z[f"U_{u}"],
                         sigma=z[f"sigma_{u}"]) for u in range(c["sweeps"] * N)]
    return c
