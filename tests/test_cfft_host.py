"""Host check of the coil-batched FFT passes' arithmetic (no GPU).

`cfft_host_check.cu` runs one pass transform serially with the kernel's own
stage index arithmetic, twiddle indices and small DFTs (the header
`pynufft_gb300/csrc/cfft_dft.cuh` the kernels include); here it is compiled
as host code with nvcc and compared with numpy.fft for every length the
passes build, forward and inverse, with the pruned input (zero padding) and
output (crop) lengths the image passes use.  Bound: 1e-6 relative L2
(float32 arithmetic lands near 1e-7).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
LENGTHS = [128, 160, 192, 256, 320, 384, 512, 640]


@pytest.fixture(scope='module')
def checker(tmp_path_factory):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('nvcc not found')
    exe = str(tmp_path_factory.mktemp('cfft') / 'cfft_host_check')
    subprocess.run([nvcc, '-std=c++17', '-O1', '-o', exe, os.path.join(HERE, 'cfft_host_check.cu')],
                   check=True, capture_output=True)
    return exe


def _run(exe, L, x, lout, inv):
    text = f'{L} {len(x)} {lout} {int(inv)}\n' + '\n'.join(f'{v.real:.9e} {v.imag:.9e}' for v in x)
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout
    a = np.array([[float(t) for t in line.split()] for line in out.strip().splitlines()])
    return a[:, 0] + 1j * a[:, 1]


@pytest.mark.parametrize('L', LENGTHS)
def test_pass_transform_matches_numpy(checker, L):
    rng = np.random.default_rng(L)
    for lin, lout, inv in [(L // 2, L, False), (L, L // 2, True), (L, L, False), (L, L, True),
                           (3 * L // 8, L, False), (L, 5 * L // 8, True)]:
        x = (rng.standard_normal(lin) + 1j * rng.standard_normal(lin)).astype(np.complex64)
        xp = np.zeros(L, np.complex128)
        xp[:lin] = x
        ref = (np.fft.ifft(xp) * L if inv else np.fft.fft(xp))[:lout]
        got = _run(checker, L, x, lout, inv)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-6, (L, lin, lout, inv, err)
