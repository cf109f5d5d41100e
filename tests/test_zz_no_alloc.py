"""The allocation-free MFT entry point, called through the C ABI (collected last on purpose).

hx_mft_execute_noalloc serves callers that cannot allocate device memory while
they run (real-time loops, host frameworks or plugin ABIs that pass only input
and output buffers): its scratch is a static device array inside the library.
These tests check it against hx_mft_execute with a caller workspace on two calls
in a row, on a plain FP32 plan and on a split tensor-core plan (whose scratch
holds sliced operands, float-float intermediates and split-K partials), the
split plan also against the float64 oracle; that the second call changes
neither the device's free memory nor torch's allocation count; and that a
transform whose scratch exceeds the static array is refused before any launch.
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
            allocs_before = torch.cuda.memory_stats()['allocation.all.allocated']
        rc = lib.hx_mft_execute_noalloc(plan.handle, _lib.HX_FORWARD, 3, _lib.dptr(e), _lib.dptr(out),
                                        alpha.real, alpha.imag, stream)
        _lib.check(rc, 'hx_mft_execute_noalloc')
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
            assert torch.cuda.memory_stats()['allocation.all.allocated'] == allocs_before
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


SPLIT_TOL = 1e-7  # split arithmetic (~2^-29 per operand) with the result rounded to complex64 (2^-24)


def test_noalloc_split_plan_matches_workspace_entry_point_and_oracle():
    """A split tensor-core plan through the static scratch: forward and backward, two calls in a row, equal bit for
    bit to hx_mft_execute with a caller workspace and within SPLIT_TOL of the float64 oracle."""
    from oracle import fourier as ofourier
    lib = _lib.lib()
    _lib.autotune(False)  # one tile choice for every call, so both entry points run the same kernels
    pupil = hg.make_pupil_grid(160, 1)
    focal = hg.make_focal_grid(4, 12)  # 96^2: small output GEMMs take the split-K partials and counters
    mft = hg.MatrixFourierTransform(pupil, focal, precision='split')
    plan = mft._plan(torch.complex64)
    batch = 2
    need = lib.hx_mft_workspace_bytes(plan.handle, _lib.HX_FORWARD, batch)
    assert 0 < need <= 16 * 1024 * 1024
    rng = np.random.default_rng(44)
    e = (rng.standard_normal((batch, pupil.size)) + 1j * rng.standard_normal((batch, pupil.size))).astype(np.complex64)
    f = (rng.standard_normal((batch, focal.size)) + 1j * rng.standard_normal((batch, focal.size))).astype(np.complex64)
    x, y = pupil.separated_coords
    u, v = focal.separated_coords
    w_in = float(np.asarray(pupil.weights).ravel()[0])
    w_out = float(np.asarray(focal.weights).ravel()[0])
    stream = _lib.stream_handle()
    cases = [(_lib.HX_FORWARD, e, focal.size, complex(w_in),
              [ofourier.mft_forward(e[i].astype(complex), x, y, u, v, w_in) for i in range(batch)]),
             (_lib.HX_BACKWARD, f, pupil.size, complex(w_out / (2 * np.pi)**2),
              [ofourier.mft_backward(f[i].astype(complex), x, y, u, v, w_out) for i in range(batch)])]
    for direction, inp, n_out, alpha, refs in cases:
        src = torch.from_numpy(inp).cuda()
        nbytes = lib.hx_mft_workspace_bytes(plan.handle, direction, batch)
        ws = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
        expect = torch.empty((batch, n_out), dtype=torch.complex64, device='cuda')
        _lib.check(lib.hx_mft_execute(plan.handle, direction, batch, _lib.dptr(src), _lib.dptr(expect), alpha.real,
                                      alpha.imag, _lib.dptr(ws), nbytes, stream))
        for call in range(2):
            out = torch.empty((batch, n_out), dtype=torch.complex64, device='cuda')
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            allocs_before = torch.cuda.memory_stats()['allocation.all.allocated']
            rc = lib.hx_mft_execute_noalloc(plan.handle, direction, batch, _lib.dptr(src), _lib.dptr(out),
                                            alpha.real, alpha.imag, stream)
            _lib.check(rc, 'hx_mft_execute_noalloc')
            torch.cuda.synchronize()
            if call == 1:
                assert torch.cuda.mem_get_info()[0] == free_before
                assert torch.cuda.memory_stats()['allocation.all.allocated'] == allocs_before
            assert torch.equal(out, expect), (direction, call)
            got = out.cpu().numpy()
            for i in range(batch):
                err = np.linalg.norm(got[i] - refs[i]) / np.linalg.norm(refs[i])
                assert err < SPLIT_TOL, (direction, call, i, err)
    assert mft._plan(torch.complex64).status() == 0


def test_noalloc_refuses_a_split_plan_beyond_the_static_scratch():
    """The headline coronagraph's 2048^2 -> 512^2 split transform needs more scratch than the static array holds
    even for one field: refused with HX_ERR_INVALID and a message, and nothing launched."""
    lib = _lib.lib()
    pupil = hg.make_pupil_grid(2048, 1)
    focal = hg.make_focal_grid(8, 32).scaled(2 * np.pi)
    mft = hg.MatrixFourierTransform(pupil, focal, precision='split')
    plan = mft._plan(torch.complex64)
    assert lib.hx_mft_workspace_bytes(plan.handle, _lib.HX_FORWARD, 1) > 16 * 1024 * 1024
    e = torch.zeros(pupil.size, dtype=torch.complex64, device='cuda')
    out = torch.zeros(focal.size, dtype=torch.complex64, device='cuda')
    before = _lib.launch_count()
    rc = lib.hx_mft_execute_noalloc(plan.handle, _lib.HX_FORWARD, 1, _lib.dptr(e), _lib.dptr(out), 1.0, 0.0,
                                    _lib.stream_handle())
    assert rc == _lib.HX_ERR_INVALID
    assert b'static scratch' in lib.hx_last_error()
    assert _lib.launch_count() == before
