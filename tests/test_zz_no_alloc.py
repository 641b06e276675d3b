"""rcwa_gpu_eig_batch_static, the eigensolver entry point that allocates nothing, against
rcwa_gpu_eig_batch_dev on the same device inputs: two calls in a row (different sizes, the second
close to the fixed workspace's limit), every lane-group form the fixed workspace can reach, the
RCWA_GB300_EIG_GROUP override honoured by both entry points alike, the oversize rejection, and no
change in free device memory across a call once the device is set up. Named to be collected last; it
also passes alone."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RCWA_OK = 0
RCWA_ESCRATCH = -5
SCRATCH_BYTES = 64 << 20


def workspace_bytes(n):
    return 16 * (3 * n * n + 4 * n + 8)


def rcwa_matrices(n, batch, seed):
    """Toeplitz permittivity matrices of a lossy binary grating with a diagonal k_x^2 shift, the
    matrices the TE eigenproblem gives."""
    rng = np.random.default_rng(seed)
    M = n // 2
    h = np.subtract.outer(np.arange(n), np.arange(n))
    out = np.empty((batch, n, n), np.complex128)
    for b in range(batch):
        e1 = complex(rng.uniform(1.3, 2.2), rng.uniform(0.0, 0.2)) ** 2
        fill = rng.uniform(0.2, 0.6)
        with np.errstate(invalid="ignore", divide="ignore"):
            eps = np.where(h == 0, fill * e1 + (1 - fill), (e1 - 1.0) * np.sin(np.pi * h * fill) / (np.pi * h))
        kx = rng.uniform(-0.5, 0.5) + (np.arange(n) - M) * 0.61
        out[b] = -eps + np.diag(kx * kx)
    return out


@pytest.fixture(scope="module")
def env(monkeypatch_module):
    import torch
    from stablercwa_gb300.engine import Engine, load_library
    monkeypatch_module.delenv("RCWA_GB300_EIG_GROUP", raising=False)
    L = load_library()
    f = L.rcwa_gpu_eig_batch_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    eng = Engine()
    yield torch, eng, f
    eng.close()


@pytest.fixture(scope="module")
def monkeypatch_module():
    mp = pytest.MonkeyPatch()
    yield mp
    mp.undo()


def device_problem(torch, n, batch, seed):
    a = rcwa_matrices(n, batch, seed)
    cm = np.ascontiguousarray(a.transpose(0, 2, 1))  # column-major storage, as the C ABI expects
    d_a = torch.from_numpy(cm).to("cuda")
    return a, d_a


def outputs(torch, n, batch):
    return (torch.empty((batch, n), dtype=torch.complex128, device="cuda"),
            torch.empty((batch, n, n), dtype=torch.complex128, device="cuda"),
            torch.empty(batch, dtype=torch.int32, device="cuda"),
            torch.empty(batch, dtype=torch.int32, device="cuda"))


def run_static(torch, f, n, batch, d_a, out):
    w, v, info, sweeps = out
    rc = f(torch.cuda.current_stream().cuda_stream, n, batch, d_a.data_ptr(), float(np.finfo(np.float64).eps), 30,
           w.data_ptr(), v.data_ptr(), info.data_ptr(), sweeps.data_ptr())
    torch.cuda.synchronize()
    return rc


def run_existing(torch, eng, n, batch, d_a):
    out = outputs(torch, n, batch)
    torch.cuda.synchronize()
    eng.eig_batch_device(n, batch, d_a.data_ptr(), out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                         out[3].data_ptr())
    eng.synchronize()
    return [t.cpu().numpy() for t in out]


def check_same(a, got, ref):
    w, v, info, sweeps = got
    w0, v0, info0, sweeps0 = ref
    assert np.all(info == 0) and np.array_equal(info, info0)
    assert np.array_equal(sweeps, sweeps0)
    scale = np.max(np.abs(w0), axis=1, keepdims=True)
    assert np.max(np.abs(w - w0) / scale) <= 1e-13
    assert np.max(np.abs(v - v0)) <= 1e-12
    V = v.transpose(0, 2, 1)  # columns are the eigenvectors
    for k in range(a.shape[0]):
        d = a[k] @ V[k] - V[k] * w[k][None, :]
        res = np.max(np.linalg.norm(d, axis=0) / (np.linalg.norm(a[k]) * np.linalg.norm(V[k], axis=0)))
        assert res <= 1e-13


def test_static_matches_existing_twice(env):
    torch, eng, f = env
    cases = [(81, 48, 1), (121, SCRATCH_BYTES // workspace_bytes(121), 2)]  # second: 94 matrices, 99.5% of the array
    problems = [(n, batch) + device_problem(torch, n, batch, seed) for n, batch, seed in cases]
    refs = [run_existing(torch, eng, n, batch, d_a) for n, batch, a, d_a in problems]
    outs = [outputs(torch, n, batch) for n, batch, _, _ in problems]
    torch.cuda.synchronize()

    # first call: sets up this device (scratch address, kernels)
    n, batch, a, d_a = problems[0]
    assert run_static(torch, f, n, batch, d_a, outs[0]) == RCWA_OK
    check_same(a, [t.cpu().numpy() for t in outs[0]], refs[0])

    # second call, right after: must not touch free device memory
    free_before = torch.cuda.mem_get_info()[0]
    n, batch, a, d_a = problems[1]
    assert run_static(torch, f, n, batch, d_a, outs[1]) == RCWA_OK
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before
    check_same(a, [t.cpu().numpy() for t in outs[1]], refs[1])


def test_static_rejects_oversize(env):
    torch, eng, f = env
    n = 121
    batch = SCRATCH_BYTES // workspace_bytes(n) + 1
    # checked on the host before anything is launched, so the pointers are never read
    dummy = torch.empty(1, dtype=torch.complex128, device="cuda")
    p = dummy.data_ptr()
    rc = f(torch.cuda.current_stream().cuda_stream, n, batch, p, float(np.finfo(np.float64).eps), 30, p, p, p, None)
    assert rc == RCWA_ESCRATCH
    n_big = 1200  # one matrix alone exceeds the array
    assert workspace_bytes(n_big) > SCRATCH_BYTES
    rc = f(torch.cuda.current_stream().cuda_stream, n_big, 1, p, float(np.finfo(np.float64).eps), 30, p, p, p, None)
    assert rc == RCWA_ESCRATCH


def default_group(n, batch):
    """The lanes per matrix both entry points choose (eig_default_group in csrc/eig.cu)."""
    lanes_wanted = 152 * 4 * 32 * 2
    for g in (4, 8, 16):
        if batch * g >= lanes_wanted and n >= 4 * g:
            return g
    if batch * 16 >= lanes_wanted:
        return 16
    if n < 64:
        return 32
    if n >= 384:
        if batch <= 152:
            return 256
        return 128 if batch * 32 < 2 * lanes_wanted else 32
    return 32 if batch * 32 * 4 >= lanes_wanted else 128


# one case per kernel form the 64 MiB workspace can hold (groups 4 and 8 need more matrices than fit):
# lane groups of 16 and 32, a CTA of 128 and of 256 threads per matrix, and one cluster per matrix (-1),
# which a few matrices of order >= 384 take by default
GROUP_CASES = [(8, 4096, 16, None), (40, 64, 32, None), (121, 94, 128, None), (400, 4, 256, "256"),
               (400, 4, -1, None)]


@pytest.mark.parametrize("n,batch,group,forced", GROUP_CASES)
def test_static_matches_existing_per_group(env, monkeypatch, n, batch, group, forced):
    torch, eng, f = env
    if forced:
        monkeypatch.setenv("RCWA_GB300_EIG_GROUP", forced)  # both entry points read it at call time
    elif group > 0:
        assert default_group(n, batch) == group
    assert batch * workspace_bytes(n) <= SCRATCH_BYTES
    a, d_a = device_problem(torch, n, batch, 10 + group)
    ref = run_existing(torch, eng, n, batch, d_a)
    out = outputs(torch, n, batch)
    assert run_static(torch, f, n, batch, d_a, out) == RCWA_OK
    check_same(a, [t.cpu().numpy() for t in out], ref)


def test_static_honours_group_override(env, monkeypatch):
    torch, eng, f = env
    n, batch = 121, 20
    assert default_group(n, batch) == 128
    monkeypatch.setenv("RCWA_GB300_EIG_GROUP", "32")  # both entry points read it at call time
    a, d_a = device_problem(torch, n, batch, 7)
    ref = run_existing(torch, eng, n, batch, d_a)
    out = outputs(torch, n, batch)
    assert run_static(torch, f, n, batch, d_a, out) == RCWA_OK
    check_same(a, [t.cpu().numpy() for t in out], ref)
