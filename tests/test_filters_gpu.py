"""Post-filters, normalisation and the temporal filter against the FP64 oracle."""
import numpy as np
import pytest

from oracle import cpu, numpy_ref
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,ksize,sigma", [((24, 30, 36), 5, 1.0), ((17, 9, 40), 3, 0.8), ((16, 16, 16), 9, 2.0)])
def test_log_filter_vs_oracle(ctx, cuda, shape, ksize, sigma):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG

    rng = np.random.default_rng(ksize)
    vol = rng.gamma(2.0, 1.0, shape).astype(np.float32)
    got = ctx.postfilter(FBP_FILTER_LOG, torch.from_numpy(vol).to(cuda), ksize, sigma).cpu().numpy()
    want = cpu.log_filter(vol, cpu.log_weights(ksize, sigma), ksize)
    # FP32 sums of k^3 zero-sum taps (the reference's order) vs FP64.
    assert rel_l2(got, want) < 5e-6


@pytest.mark.parametrize("ksize", [3, 5])
def test_laplacian_vs_oracle(ctx, cuda, ksize):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LAPLACIAN

    vol = np.random.default_rng(1).random((21, 18, 25)).astype(np.float32)
    got = ctx.postfilter(FBP_FILTER_LAPLACIAN, torch.from_numpy(vol).to(cuda), ksize).cpu().numpy()
    assert rel_l2(got, cpu.laplacian_filter(vol, ksize)) < 1e-6


def test_postfilter_none_copies_and_rejects_aliasing(ctx, cuda):
    import torch
    from fasterbackprojection_gb300 import FBP_FILTER_LOG, FBP_FILTER_NONE, FbpError

    v = torch.rand((8, 8, 8), device=cuda)
    assert torch.equal(ctx.postfilter(FBP_FILTER_NONE, v), v)
    with pytest.raises(FbpError):
        ctx.postfilter(FBP_FILTER_LOG, v, out=v)
    with pytest.raises(FbpError):
        ctx.postfilter(FBP_FILTER_LOG, v, kernel_size=17)


@pytest.mark.parametrize("n", [1, 5, 4096, 1_234_567])
def test_normalize_vs_oracle(ctx, cuda, n):
    import torch

    v = np.random.default_rng(n).normal(size=n).astype(np.float32) * 3
    got = ctx.normalize_(torch.from_numpy(v).to(cuda)).cpu().numpy()
    want = cpu.normalize(v.astype(np.float64))
    assert np.abs(got - want).max() < 1e-6


@pytest.mark.parametrize("T,border", [(1024, "zero"), (512, "edge"), (37, "zero")])
def test_filter_h_vs_fp64_fft(ctx, cuda, T, border):
    import torch
    from fasterbackprojection_gb300 import FBP_BORDER_EDGE, FBP_BORDER_ZERO

    rng = np.random.default_rng(T)
    data = rng.poisson(2.0, (300, T)).astype(np.float32)
    step = 0.0048
    d = torch.from_numpy(data).to(cuda)
    ctx.filter_h_(d, step, border=FBP_BORDER_EDGE if border == "edge" else FBP_BORDER_ZERO)
    want = numpy_ref.filter_h(data, step, border=border)
    assert rel_l2(d.cpu().numpy(), want) < 2e-6


@pytest.mark.parametrize("wl_bins", [1.5, 3.0, 6.0, 30.0])
def test_filter_h_wavelengths_vs_fp64_fft(ctx, cuda, wl_bins):
    """Tap counts of 2 to 20 blocks of 16 (the unrolled forms and the general
    loop), against the FP64 padded-FFT pipeline."""
    import torch

    rng = np.random.default_rng(int(wl_bins * 10))
    T = 1024
    data = rng.poisson(2.0, (200, T)).astype(np.float32)
    step = 0.0048
    d = torch.from_numpy(data).to(cuda)
    ctx.filter_h_(d, step, wl_mean=wl_bins * step)
    want = numpy_ref.filter_h(data, step, wl_mean=wl_bins * step)
    assert rel_l2(d.cpu().numpy(), want) < 2e-6


def test_filter_h_vs_reference_fft_pipeline(ctx, cuda):
    """Against the reference's own arithmetic path on the GPU: padded series,
    batched C2C FFT (cuFFT through torch), the spectrum product, unnormalised
    inverse, real part of the unpadded bins (Laser.cu:174-234)."""
    import torch

    rng = np.random.default_rng(99)
    T = 1024
    data = rng.poisson(1.5, (500, T)).astype(np.float32)
    step = 0.0048
    sigma, t6, n = numpy_ref.filter_h_params(T, step, 10 * step)
    K = numpy_ref.filter_h_kernel(n, float(np.float32(step)), float(np.float32(10 * step)), sigma)
    pad = (n - T) // 2
    H = torch.zeros((500, n), dtype=torch.complex64, device=cuda)
    H[:, pad:pad + T] = torch.from_numpy(data).to(cuda)
    Kt = torch.from_numpy(K.astype(np.complex64)).to(cuda)
    ref = torch.fft.ifft(torch.fft.fft(H, dim=1) * torch.fft.fft(Kt)[None], dim=1, norm="forward")
    ref = ref[:, pad:pad + T].real.cpu().numpy()
    d = torch.from_numpy(data).to(cuda)
    ctx.filter_h_(d, step)
    assert rel_l2(d.cpu().numpy(), ref) < 2e-5
