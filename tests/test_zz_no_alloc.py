"""falcon_download_state_range: the allocation-free state download.

It is called through the C ABI and checked against falcon_download_state on
the same device state. Widening FP32 to FP64 is exact, so the tolerance is
zero: the two downloads must be bit-identical. The range call stages through a
static device array shared by every call, so the test makes two whole-state
downloads in a row (checking that neither depends on what the previous call
left there), and one more after the state has changed.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import falcon_gb300 as fg
from falcon_gb300 import config

pytestmark = pytest.mark.gpu

MAX_ELEMS = fg.STATIC_SCRATCH_BYTES // 8


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib):
    return built_lib


def _cudart():
    """The CUDA runtime as a shared library, for an independent reading of the
    device's free memory (the library under test links its own runtime)."""
    root = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for p in sorted(glob.glob(os.path.join(root, "lib64", "libcudart.so*")) +
                    glob.glob(os.path.join(root, "targets", "*", "lib", "libcudart.so*"))):
        try:
            return C.CDLL(p)
        except OSError:
            continue
    return None


def _free_bytes(rt):
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _range_call(f, first, count, out):
    return fg.lib().falcon_download_state_range(f.h, C.c_size_t(first), C.c_size_t(count),
                                                out.ctypes.data_as(C.c_void_p))


def _download_by_ranges(f, chunk):
    out = np.full(f.shape, np.nan)
    flat = out.reshape(-1)
    first = 0
    while first < flat.size:
        count = min(chunk, flat.size - first)
        rc = _range_call(f, first, count, flat[first:])
        assert rc == fg.OK, f.last_error()
        first += count
    return out


@pytest.mark.parametrize("prec", [config.PREC_MIXED, config.PREC_FP64])
def test_range_download_matches_download_state(prec):
    # 864 blocks x 8 variables x 12^3 cells = 11.9M elements: several full ranges
    f = fg.Falcon(config.shell_fp64_cpu(precision=prec, device=0))
    assert f.shape[0] * np.prod(f.shape[1:]) > 2 * MAX_ELEMS
    f.init_synthetic(kind=1, seed=2024, mach=0.05)
    f.exchange()
    before = f.device_bytes()
    a = _download_by_ranges(f, MAX_ELEMS)
    _download_by_ranges(f, 1_000_003)
    # free device memory read through the CUDA runtime after a first round of
    # both chunk shapes (which may load the library's device code and set up
    # the driver's copy paths for these sizes): a cudaMalloc on any path of the
    # range call, the context's allocator or not, would lower it
    rt = _cudart()
    free0 = _free_bytes(rt) if rt is not None else None
    b = _download_by_ranges(f, 1_000_003)          # ragged ranges
    a2 = _download_by_ranges(f, MAX_ELEMS)         # whole ranges, second call in a row
    assert f.device_bytes() == before              # the range calls allocated nothing
    if rt is not None:
        assert _free_bytes(rt) == free0
    assert np.array_equal(a2, a)
    ref = f.download_state()
    assert np.array_equal(a, ref)
    assert np.array_equal(b, ref)
    # the state changes; the next range download follows it
    f.advance_rk4()
    ref2 = f.download_state()
    assert not np.array_equal(ref2, ref)
    c = _download_by_ranges(f, MAX_ELEMS)
    assert np.array_equal(c, ref2)


def test_range_download_rejects_oversize_and_out_of_range():
    f = fg.Falcon(config.tiny(precision=config.PREC_MIXED, device=0))
    n = int(np.prod(f.shape))
    out = np.full(MAX_ELEMS + 1, -7.0)
    assert _range_call(f, 0, MAX_ELEMS + 1, out) == fg.ERR_INVALID_ARG
    assert "static scratch limit" in f.last_error()
    assert _range_call(f, n - 10, 11, out) == fg.ERR_INVALID_ARG
    assert "exceeds the state size" in f.last_error()
    assert (out == -7.0).all()                     # rejected calls leave u untouched
    assert _range_call(f, n, 0, out) == fg.OK      # empty range at the end
