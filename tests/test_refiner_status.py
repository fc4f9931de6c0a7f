"""A tensor-core wait that gives up reaches the caller as an error.

CPU: the status call of the C-ABI is replaced by a fake that reports
TDE_ERR_DEVICE_TIMEOUT (the failure is made on the host, no GPU involved);
Refiner.status() returns the code and Refiner.check_status() raises TdeError
with it, as the benchmark and the training loop rely on.
GPU: the bounded wait the refiner kernels use, run on its own against a
barrier phase nothing completes (tde_wait_selftest), gives up after its limit
and raises the flag; the context keeps working."""
import ctypes as C
import importlib

import pytest


class _FakeLib:
    """The refiner's C-ABI calls with a status call that reports a device timeout."""

    def __init__(self, lib):
        self._lib = lib

    def tde_refiner_status(self, handle):
        return -4  # TDE_ERR_DEVICE_TIMEOUT

    def tde_last_error(self):
        return b"refiner: a tensor-core wait timed out"

    def __getattr__(self, name):
        return getattr(self._lib, name)


def test_status_timeout_surfaces_as_error(tde, monkeypatch):
    rf = importlib.import_module("3deye_gb300.refiner")
    capi = importlib.import_module("3deye_gb300._capi")
    fake = _FakeLib(capi.lib)
    monkeypatch.setattr(rf, "lib", fake)
    monkeypatch.setattr(capi, "lib", fake)
    R = rf.Refiner.__new__(rf.Refiner)  # no device state: only the status path runs
    R._h = C.c_void_p(1)
    assert R.status() == capi.TDE_ERR_DEVICE_TIMEOUT
    with pytest.raises(capi.TdeError) as e:
        R.check_status()
    assert e.value.code == capi.TDE_ERR_DEVICE_TIMEOUT and "timed out" in str(e.value)
    R._h = None  # nothing to destroy


def test_selftest_arguments_refused_on_host(tde):
    importlib.import_module("3deye_gb300.refiner")
    assert tde.lib.tde_wait_selftest(1000, None, None) == -1
    assert tde.lib.tde_wait_selftest(0, C.c_void_p(8), None) == -1


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_context_survives(tde, cuda):
    import torch
    importlib.import_module("3deye_gb300.refiner")
    out = torch.zeros(2, dtype=torch.int64, device=cuda)
    tde.check(tde.lib.tde_wait_selftest(2_000_000, out.data_ptr(), tde.stream_ptr()))  # 2 ms
    torch.cuda.synchronize()
    flag, waited = (int(v) for v in out.cpu())
    assert flag == 1
    assert 2_000_000 <= waited < 1_000_000_000
    # the context is usable afterwards
    x = torch.arange(1000, device=cuda, dtype=torch.float32)
    assert float(x.sum().item()) == 499500.0
