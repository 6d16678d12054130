import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "grazelle-ppopp18_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    """(record dict, EdgeList) of a golden case; generated graphs are regenerated from their seed."""
    from grazelle import graphgen as gg
    rec = dict(np.load(GOLDEN / (name + ".npz")))
    V = int(rec["V"])
    if "pairs_pull" in rec:
        p = rec["pairs_pull"]
        g = gg.EdgeList(V, p[0::2].copy(), p[1::2].copy())
    else:
        kind = str(rec["spec_kind"])
        if kind == "rmat":
            g = gg.rmat(int(rec["spec_scale"]), int(rec["spec_edge_factor"]), seed=int(rec["spec_seed"]))
        elif kind == "rmat_sym":
            g = gg.symmetrize(gg.rmat(int(rec["spec_scale"]), int(rec["spec_edge_factor"]), seed=int(rec["spec_seed"])))
        elif kind == "er":
            g = gg.erdos_renyi(int(rec["spec_n"]), float(rec["spec_avg_degree"]), seed=int(rec["spec_seed"]))
        else:
            raise ValueError(kind)
    assert g.num_edges == int(rec["E"]), "regenerated graph differs from the fixture"
    return rec, g


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
