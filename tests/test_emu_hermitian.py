"""The Hermitian eigensolver's CUDA kernels (stablercwa_gb300/csrc/eig.cuh) compiled for the host and run
through a thread-level emulation of the CUDA primitives they use (tests/emu/): the tridiagonalisation with
4..32 lanes per matrix, the QL kernel with d and e in shared memory and in the workspace, and the rotations
applied to a real identity or to the complex Q, on random Hermitian, Toeplitz-plus-Kx^2 and diagonal
(repeated-eigenvalue) matrices of orders 1..61 and on symmetric-Toeplitz, Wilkinson W+ and glued matrices
(clustered spectra) of orders 1..162, and lossless high-contrast grating layer matrices of order 301
(M = 150; ridge index 3.48 and 4.0 in air, TE and the TM pencil matrix with its explicit L^-1) on the
128-thread CTA form a lone solve of that order takes and on the blocked form with 32 and 16 lanes; the fixed-point rotation product alone on synthetic sweeps of
orders 2..301 against long-double arithmetic (max |Y - exact| <= 2e-16), and the conversion of rotation
coefficients to that fixed point on 200,000 values and its edge cases; the blocked reduction (herm_panel_one, panels of 32
reflectors, the trailing update and the back-transformation X = Q Y from the stored reflectors and T V^H as
host products) at orders 64, 65, 97 and 121 (partial and full last panels); the divide-and-conquer
tridiagonal eigensolver (herm_dc_one) at orders 1..162 on random, Toeplitz-plus-Kx^2, diagonal (massive
deflation), Wilkinson W+ (eigenvalue pairs equal to many digits) and glued (clusters) matrices; and the
general solver (eig_one, 4 and 32 lanes and a
64-thread CTA) on random complex matrices of orders 1..30. Eigenpair residuals <= 1e-13, orthonormal
columns for the Hermitian solver. This checks the kernels' arithmetic and index logic without a GPU; the
device runs are the -m gpu tests."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_hermitian_kernels_in_emulation(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "herm_emu"
    build = subprocess.run([cxx, "-O2", "-std=c++20", "-pthread", "-I", os.path.join(HERE, "emu"), "-o", str(exe),
                            os.path.join(HERE, "emu", "herm_emu.cpp")], capture_output=True, text=True, timeout=300)
    assert build.returncode == 0, build.stderr[-2000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=900)
    assert run.returncode == 0 and run.stdout.strip().endswith("OK"), run.stdout[-3000:]
    assert run.stdout.count("pass ") == 151
