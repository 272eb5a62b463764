import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))

CASES = ["pbm_pbmclicks", "ubm_dbnclicks", "dbn_dbnclicks", "ccm_ccmclicks", "dbn_ccmclicks", "edge"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_case(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def case_models(case: dict) -> list[int]:
    return [int(m) for m in case["models"]]


def dumped_iters(case: dict, model: int) -> list[int]:
    its = []
    for k in case:
        if k.startswith(f"m{model}_params_"):
            its.append(int(k.split("_")[-1]))
    return sorted(its)


@pytest.fixture(scope="session")
def native_lib():
    from massiveclicks_gb300 import _capi
    return _capi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import bindings
    return bindings.load()


def cuda_available() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            from massiveclicks_gb300 import _capi
            _capi.load()
            import ctypes
            rt = ctypes.CDLL("libcudart.so.13")
        except OSError:
            return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
