"""The allocation-free MFT entry point, called through the C ABI (collected last on purpose).

hx_mft_execute_noalloc serves callers that cannot allocate device memory while
they run (real-time loops, host frameworks or plugin ABIs that pass only input
and output buffers): its scratch is a static device array inside the library.
This test checks it against hx_mft_execute with a caller workspace on two calls
in a row, that the second call changes the device's free memory by nothing, and
that a batch larger than the static scratch is refused before any launch.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

hg = pytest.importorskip('hcipy_gb300')
from hcipy_gb300 import _lib  # noqa: E402

TOL32 = 3e-6  # the float32 MFT tolerance used by the other device tests


def _plan_and_fields(batch):
    pupil = hg.make_pupil_grid(256, 1)
    focal = hg.make_focal_grid(4, 16)
    mft = hg.MatrixFourierTransform(pupil, focal)
    rng = np.random.default_rng(12)
    e = (rng.standard_normal((batch, pupil.size)) + 1j * rng.standard_normal((batch, pupil.size))).astype(np.complex64)
    e = torch.from_numpy(e).cuda()
    plan = mft._plan(torch.complex64)
    return mft, plan, e, focal


def test_noalloc_matches_workspace_entry_point():
    lib = _lib.lib()
    mft, plan, e, focal = _plan_and_fields(batch=3)
    alpha = complex(mft._w_in_scalar)
    ref = mft.forward(e).data
    torch.cuda.synchronize()
    stream = _lib.stream_handle()
    outs = []
    free_before = None
    for call in range(2):
        out = torch.empty((3, focal.size), dtype=torch.complex64, device='cuda')
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = lib.hx_mft_execute_noalloc(plan.handle, _lib.HX_FORWARD, 3, _lib.dptr(e), _lib.dptr(out),
                                        alpha.real, alpha.imag, stream)
        _lib.check(rc, 'hx_mft_execute_noalloc')
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        outs.append(out)
    for out in outs:
        err = (torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item()
        assert err < TOL32
    # The backward direction uses the same scratch.
    f = mft.forward(e).data
    back_ref = mft.backward(f).data
    back = torch.empty_like(e)
    a_b = complex(mft._w_out_scalar / (2 * np.pi)**2)
    rc = lib.hx_mft_execute_noalloc(plan.handle, _lib.HX_BACKWARD, 3, _lib.dptr(f), _lib.dptr(back), a_b.real,
                                    a_b.imag, stream)
    _lib.check(rc)
    torch.cuda.synchronize()
    assert (torch.linalg.norm(back - back_ref) / torch.linalg.norm(back_ref)).item() < TOL32


def test_noalloc_rejects_batches_beyond_the_static_scratch():
    lib = _lib.lib()
    mft, plan, e, focal = _plan_and_fields(batch=1)
    per_field = lib.hx_mft_workspace_bytes(plan.handle, _lib.HX_FORWARD, 1)
    too_many = (16 * 1024 * 1024) // per_field + 1
    before = _lib.launch_count()
    rc = lib.hx_mft_execute_noalloc(plan.handle, _lib.HX_FORWARD, too_many, _lib.dptr(e), _lib.dptr(e), 1.0, 0.0,
                                    _lib.stream_handle())
    assert rc == _lib.HX_ERR_INVALID
    assert b'static scratch' in lib.hx_last_error()
    assert _lib.launch_count() == before
