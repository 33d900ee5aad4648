"""The tensor-core probe of the z-transform (tests/ozaki_probe.py): the bf16
digit products are exact in FP32 accumulation, and the split product
reproduces the FP64 backward z-DFT of the benchmark box's columns to 1e-14 of
the largest output (seven 8-bit digits)."""
import numpy as np
import pytest

import ozaki_probe as oz

pytestmark = pytest.mark.gpu


def _mm_or_skip():
    import torch
    a = torch.ones((2, 2), dtype=torch.bfloat16, device="cuda")
    try:
        torch.mm(a, a, out_dtype=torch.float32)
    except (TypeError, RuntimeError) as e:  # older torch: no bf16 -> fp32 product
        pytest.skip(f"torch.mm(out_dtype=float32) unavailable: {e}")


def test_digit_products_are_exact():
    import torch
    _mm_or_skip()
    rng = np.random.default_rng(1)
    a = rng.integers(-128, 129, (192, 126)).astype(np.float64)
    b = rng.integers(-128, 129, (126, 4096)).astype(np.float64)
    got = oz.mm32(torch.tensor(a, device="cuda").to(torch.bfloat16),
                  torch.tensor(b, device="cuda").to(torch.bfloat16))
    assert np.array_equal(got.double().cpu().numpy(), a @ b)


def test_split_product_matches_fp64_dft():
    import torch
    _mm_or_skip()
    A = torch.tensor(oz.dft_block(), device="cuda")
    Xh = oz.columns()[:, :8192]
    X = torch.tensor(Xh, device="cuda")
    Y = oz.ozaki_product(A, X, 7).cpu().numpy()
    # the backward transform of the same columns by numpy's FFT (zero-filled
    # 2/3-rule modes, unnormalised)
    C = Xh[:oz.MZ] + 1j * Xh[oz.MZ:]
    full = np.zeros((oz.MGALZ, C.shape[1]), complex)
    full[:oz.NZ + 1] = C[:oz.NZ + 1]
    full[oz.MGALZ - oz.NZ:] = C[oz.NZ + 1:]
    ref = np.fft.ifft(full, axis=0) * oz.MGALZ
    want = np.concatenate([ref.real, ref.imag], axis=0)
    assert np.abs(Y - want).max() <= 1e-14 * np.abs(want).max()
