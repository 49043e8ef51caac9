"""The tensor-core Gram-Schmidt projection H = V^T W (tcgen05 kind::tf32
with the 3xTF32 split, TMA-fed; nm_gs_tc.cu) against the same product in
FP64, through the library's test hook.

The split product has a relative error of about 2^-21 per term, so every
entry is held to 4e-6 of |v_k| |w_c| (the Cauchy-Schwarz bound of the sum);
plain FP32 accumulation over 1e5 terms is of the same order.  Row counts
that are not a multiple of the 32-row stage exercise the zero-filled TMA
tail; K = 64 runs a tile whose second 64-column chunk is absent."""
import numpy as np
import pytest

from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


@pytest.mark.parametrize("n,K", [(100003, 256), (4099, 64), (262144, 1024)])
def test_tensor_core_projection_matches_fp64(n, K):
    import torch
    from normalmodes_gb300 import nmgpu
    L = nmgpu.lib()
    ld = (n + 31) // 32 * 32
    g = torch.Generator(device="cuda").manual_seed(5)
    V = torch.zeros((K, ld), dtype=torch.float32, device="cuda")  # column-major n x K, leading dimension ld
    V[:, :n] = torch.randn((K, n), generator=g, device="cuda")
    W = torch.zeros((32, ld), dtype=torch.float32, device="cuda")
    W[:, :n] = torch.randn((32, n), generator=g, device="cuda")
    H = torch.full((32, K), float("nan"), dtype=torch.float32, device="cuda")  # column-major K x 32, ld K
    torch.cuda.synchronize()
    rc = L.nm_test_gs_tc(V.data_ptr(), ld, n, K, W.data_ptr(), ld, H.data_ptr(), K)
    assert rc == 0, rc
    torch.cuda.synchronize()
    ref = (V[:, :n].double() @ W[:, :n].double().T)  # K x 32
    got = H.double().T
    scale = V[:, :n].double().norm(dim=1)[:, None] * W[:, :n].double().norm(dim=1)[None, :]
    err = ((got - ref).abs() / scale).max().item()
    f32 = ((V[:, :n] @ W[:, :n].T).double() - ref).abs().div(scale).max().item()
    print(f"n={n} K={K}: tensor-core 3xTF32 rel err {err:.2e} (FP32 matmul {f32:.2e})")
    assert np.isfinite(err) and err <= 4e-6
