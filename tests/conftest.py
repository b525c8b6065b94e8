import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "gal-dawn_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libdawn_gb300.so)")


class Golden:
    """One committed fixture: the CSR the reference loader built from the
    .mtx beside it, and the reference tools' outputs for a few sources."""

    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.basename(path)[:-4]
        self.mtx = path[:-4] + ".mtx"
        self.n = int(z["n"])
        self.row_ptr = z["row_ptr"]
        self.col = z["col"]
        self.directed = bool(z["directed"])
        self.symmetric = not self.directed
        self.weighted = bool(z["weighted"])
        self.w_f32 = z["val"] if "val" in z.files else None
        self.w_i32 = self.w_f32.astype(np.int32) if self.w_f32 is not None else None
        self.sources = z["sources"]
        self.bfs_ref = z["bfs_ref"]
        self.bfs_text0 = str(z["bfs_text0"])
        self.cc_text = [str(x) for x in z["cc_text"]]
        self.sssp_ref = z["sssp_ref"] if "sssp_ref" in z.files else None
        self.sssp_text0 = str(z["sssp_text0"]) if "sssp_text0" in z.files else None
        self.ccw_text = [str(x) for x in z["ccw_text"]] if "ccw_text" in z.files else None
        self.mssp_sources = z["mssp_sources"] if "mssp_sources" in z.files else None
        self.mssp_ref = z["mssp_ref"] if "mssp_ref" in z.files else None

    @property
    def m(self):
        return int(self.col.shape[0])

    def degrees(self):
        return np.diff(self.row_ptr.astype(np.int64))


def golden_all():
    return [Golden(p) for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))]


@pytest.fixture(scope="session")
def goldens():
    gs = golden_all()
    assert gs, "no golden fixtures"
    return gs


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
