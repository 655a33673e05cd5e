"""The reference's continuation calls cufftExecZ2D on half spectra whose
self-conjugate bins are not Hermitian (UpContinuation_gpu.cu:113-164,244-248).
The oracle (and the CUDA path) model that call as the inverse DFT of the
Hermitian part of the spectrum; this test runs cuFFT itself on seeded
non-Hermitian inputs at even and odd sizes and checks that model."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SIZES = [(12, 10), (13, 11), (44, 46), (260, 435), (736, 736)]


def projection_c2r(X, M1, L1):
    H = L1 // 2 + 1
    G = np.fft.ifft(X, axis=0) * M1
    full = np.zeros((M1, L1), complex)
    full[:, :H] = G
    full[:, 0] = G[:, 0].real
    if L1 % 2 == 0:
        full[:, L1 // 2] = G[:, L1 // 2].real
    for kx in range(1, (L1 + 1) // 2):
        full[:, L1 - kx] = np.conj(G[:, kx])
    return np.fft.ifft(full, axis=1).real * L1


def test_cufft_z2d_is_the_hermitian_projection(tmp_path):
    exe = str(tmp_path / "probe")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                    os.path.join(HERE, "cufft_c2r_probe.cu"), "-lcufft"], check=True)
    args = [str(v) for mn in SIZES for v in mn]
    subprocess.run([exe, str(tmp_path)] + args, check=True)
    for M1, L1 in SIZES:
        b = open(tmp_path / f"c2r_{M1}_{L1}.bin", "rb").read()
        H = L1 // 2 + 1
        X = np.frombuffer(b[8:8 + M1 * H * 16], np.complex128).reshape(M1, H)
        Y = np.frombuffer(b[8 + M1 * H * 16:], np.float64).reshape(M1, L1)
        P = projection_c2r(X, M1, L1)
        assert np.abs(Y - P).max() <= 1e-13 * np.abs(Y).max(), (M1, L1)
