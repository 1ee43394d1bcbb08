"""Device-side failure detection without a GPU fault: a bounded wait that
runs out reports GBF_ERR_TIMEOUT and the context stays usable; a non-finite
input is reported through the status word (host-injected)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(gpu_lib, abi, pkg, O, oracle):
    ms = ctypes.c_double()
    for tries in (1 << 10, 1 << 14):
        assert gpu_lib.gbf_diag_bounded_wait(tries, ctypes.byref(ms)) == abi.GBF_ERR_TIMEOUT
        assert ms.value < 5000.0
        print(f"bounded wait, {tries} rounds: {ms.value:.3f} ms")
    gpu_lib.gbf_clear_status()
    # the context is still usable: a split step runs and stays finite
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m = abi.reference_model(16, 12, 10, 0.01)
    st = O.State(m)
    oracle.initial(st)
    dom = Domain(m, precision=abi.GBF_PREC_SPLIT_DF)
    dom.upload(st["P1"], st["S2"])
    dom.step(3)
    assert dom.status() == abi.GBF_OK
    assert np.isfinite(dom.download("S2")).all()
    dom.close()
