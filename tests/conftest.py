import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for sub in ("oracle", "eigen-git-mirror_gb300"):
    p = str(ROOT / sub)
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden" / "llt_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (sm_103)")
    config.addinivalue_line("markers", "slow: full-size case (seconds)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build(ref=False) if not O.LIB_PATH.exists() else None
    return O


@pytest.fixture(scope="session")
def gbllt():
    import gbllt as G
    return G


def load_golden():
    """List of golden cases produced by Eigen's own LLT (tests/golden/make_golden.py)."""
    z = np.load(GOLDEN)
    cases = []
    for i in range(int(z["ncases"])):
        p = f"c{i:03d}_"
        n, seed, nrhs, fail, info = (int(v) for v in z[p + "meta"])
        c = dict(kind=str(z[p + "kind"]), n=n, seed=seed, nrhs=nrhs, fail=fail, info=info,
                 dtype=str(z[p + "dtype"]), uplo=str(z[p + "uplo"]), asum=z[p + "asum"])
        if p + "factor" in z:
            c["factor"] = z[p + "factor"]
            c["x"] = z[p + "x"]
        cases.append(c)
    return cases


def golden_input(O, c):
    """Regenerate the input matrix and right-hand side of a golden case from its seeds."""
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import make_golden as MG
    a64 = MG.make_input(c["kind"], c["n"], c["seed"])
    dtype = np.float64 if c["dtype"] == "d" else np.float32
    a = np.asfortranarray(a64.astype(dtype))
    n, k = c["n"], c["nrhs"]
    b = np.asfortranarray(O.normal(2, n * k).reshape(k, n).T.astype(dtype))
    return a64, a, b


def tri(a, uplo):
    n = a.shape[0]
    idx = np.tril_indices(n) if uplo == "L" else np.triu_indices(n)
    return a[idx]


def rel(x, y):
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    d = np.linalg.norm(y)
    return float(np.linalg.norm(x - y) / (d if d > 0 else 1.0))
