"""The eigensolver autotuner (csrc/autotune.cu): it times every applicable kernel form on real matrices,
records the fastest for (solver, order, batch bucket), and the solves then use exactly that form: the
results of an untuned-key call after tuning equal, bit for bit, those of the same call with the form forced."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = {-1, 4, 8, 16, 32, 64, 128, 256}


def layer_matrices(n, batch, seed):
    rng = np.random.default_rng(seed)
    M = n // 2
    h = np.subtract.outer(np.arange(n), np.arange(n))
    out = np.empty((batch, n, n), np.complex128)
    for b in range(batch):
        e1 = complex(1.46, 0.01) ** 2
        fill = rng.uniform(0.3, 0.6)
        with np.errstate(invalid="ignore", divide="ignore"):
            eps = np.where(h == 0, fill * e1 + (1 - fill), (e1 - 1.0) * np.sin(np.pi * h * fill) / (np.pi * h))
        kx = rng.uniform(-0.5, 0.5) + (np.arange(n) - M) * 0.61
        out[b] = np.diag(kx * kx) - eps
    return out


@pytest.mark.parametrize("hermitian,n,batch", [(False, 45, 300), (True, 45, 300), (False, 121, 2)])
def test_tuned_form_is_used(monkeypatch, hermitian, n, batch):
    """(121, 2): a key where the thread-block cluster form is among the timed candidates."""
    import torch
    from stablercwa_gb300.engine import Engine, autotune_table
    a = layer_matrices(n, batch, 3)
    if hermitian:
        a = 0.5 * (a + a.conj().transpose(0, 2, 1))
    d_a = torch.from_numpy(np.ascontiguousarray(a.transpose(0, 2, 1))).to("cuda")
    eng = Engine()
    try:
        form, ms = eng.autotune_eig(n, batch, d_a.data_ptr(), hermitian=hermitian)
        assert form in FORMS and ms > 0
        bucket = 1 << (batch.bit_length() - 1)
        line = f"{'hermitian' if hermitian else 'general'} {n} {bucket} {form}"
        assert line in autotune_table()
        solve = eng.eig_hermitian_batch if hermitian else eng.eig_batch
        monkeypatch.delenv("RCWA_GB300_EIG_GROUP", raising=False)
        tuned = solve(a)
        monkeypatch.setenv("RCWA_GB300_EIG_GROUP", str(form))
        forced = solve(a)
        for x, y in zip(tuned[:2], forced[:2]):
            assert np.array_equal(x, y)
    finally:
        eng.close()
