"""Seeded fields generated on the device against the host generator: porosity
bit for bit; log-normal K within 1 FP32 ulp and nearly everywhere equal
(the two sides' log/cos/exp may round the last bit differently)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,corr", [((40, 36, 28), 3.0), ((17, 9, 23), 0.0), ((64, 64, 64), 8.0)])
def test_device_fields_equal_host_fields(gpu_lib, abi, shape, corr):
    import torch
    nx, ny, nz = shape
    n = nx * ny * nz
    Kh = np.empty(n, np.float32)
    ph = np.empty(n, np.float32)
    assert gpu_lib.gbf_fill_lognormal_K(nx, ny, nz, 77, 6.64e-11, 1.2, corr, Kh.ctypes.data) == 0
    assert gpu_lib.gbf_fill_porosity(nx, ny, nz, 78, 0.35, 0.05, ph.ctypes.data) == 0
    Kd = torch.empty(n, dtype=torch.float32, device="cuda")
    pd = torch.empty(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert gpu_lib.gbf_fill_lognormal_K_device(nx, ny, nz, 77, 6.64e-11, 1.2, corr, Kd.data_ptr(), None) == 0
    assert gpu_lib.gbf_fill_porosity_device(nx, ny, nz, 78, 0.35, 0.05, pd.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(pd.cpu().numpy(), ph)
    K = Kd.cpu().numpy()
    rel = np.abs(K.astype(np.float64) - Kh) / Kh
    assert rel.max() <= 2.0 ** -23
    assert (K == Kh).mean() >= 0.999
    # the statistics the generator promises
    z = np.log(Kh.astype(np.float64) / 6.64e-11)
    assert abs(z.mean()) < 1e-5 and abs(z.std(ddof=1) - 1.2) < 1e-5
