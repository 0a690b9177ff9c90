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
