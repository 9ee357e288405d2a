"""The library's own 3-D R2C FFT (power-of-two meshes) against torch.fft.rfftn
in float64 on the same float32 input.  Tolerance: norm-wise relative error
below 2e-7 * log2(N^3) (float32 round-off growth of a radix-8 FFT)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [64, 128, 256, 512])
@pytest.mark.parametrize("G", [1, 2])
def test_own_fft_matches_rfftn(N, G):
    from gbpowspec import _native
    dev = torch.device("cuda", 0)
    plan = _native.FFTPlan(N, G, dev)
    assert plan.pitch == N // 2 + 8 and plan.ws_bytes == 0
    torch.manual_seed(N + G)
    mesh = torch.randn(G, N, N, N, device=dev) + 0.3
    spec = torch.full((plan.spectrum_floats,), float("nan"), device=dev)
    plan.execute(mesh, spec)
    s = spec.view(G, N, N, plan.pitch, 2)
    got = torch.view_as_complex(s[..., : N // 2 + 1, :].contiguous()).to(torch.complex128)
    want = torch.fft.rfftn(mesh.double(), dim=(1, 2, 3))
    err = (got - want).abs().pow(2).sum().sqrt() / want.abs().pow(2).sum().sqrt()
    assert err.item() < 2e-7 * math.log2(N ** 3), err.item()
    assert torch.count_nonzero(s[..., N // 2 + 1:, :]) == 0      # row padding written as zeros
    plan.close()


def test_own_fft_matches_cufft_backend(monkeypatch):
    """The same transform through cuFFT (forced at plan creation) agrees to round-off."""
    from gbpowspec import _native
    dev = torch.device("cuda", 0)
    N = 128
    mesh = torch.randn(2, N, N, N, device=dev)
    own = _native.FFTPlan(N, 2, dev)
    monkeypatch.setenv("GBP_FFT_BACKEND", "cufft")
    cuf = _native.FFTPlan(N, 2, dev)
    assert cuf.pitch == N // 2 + 1
    a = torch.empty(own.spectrum_floats, device=dev)
    b = torch.empty(cuf.spectrum_floats, device=dev)
    own.execute(mesh, a)
    cuf.execute(mesh, b)
    ca = torch.view_as_complex(a.view(2, N, N, own.pitch, 2)[..., : N // 2 + 1, :].contiguous())
    cb = torch.view_as_complex(b.view(2, N, N, cuf.pitch, 2))
    err = ((ca - cb).abs().pow(2).sum() / cb.abs().pow(2).sum()).sqrt().item()
    assert err < 1e-6, err
    own.close()
    cuf.close()
