"""dd_fft_c2r_noalloc: the backward transform for callers that cannot
allocate device memory (their memory belongs to an application pool, or a
cudaMalloc and its implicit device synchronisation are not allowed where they
call from).  It keeps its intermediates in a 4 MiB static device buffer
instead of a caller workspace.

Checked through the C ABI against the existing entry point dd_fft_c2r (with a
workspace) on two calls in a row, with different inputs, at the FP64
transform tolerance used by the other transform tests (1e-13 relative max
error).  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,dealiasing", [((64, 64, 64), '2/3 cython'), ((32, 16, 64), '2/3 cython'),
                                              ((128, 128), '2/3 cython'), ((512, 512), '2/3 cython'),
                                              # no dealiasing: every mode but the Nyquist ones, 4.16 MB
                                              ((64, 64, 64), 'None'), ((512, 512), 'None')])
def test_noalloc_c2r_matches_workspace_c2r(dd, cuda, shape, dealiasing):
    import torch
    plan = dd.engine.Plan(shape, (2 * np.pi,) * len(shape), dealiasing=dealiasing)
    rng = np.random.default_rng(sum(shape) + 11)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        k = rng.standard_normal(plan.kshape) + 1j * rng.standard_normal(plan.kshape)
        kd = torch.from_numpy(k).to(cuda)
        x_ref = torch.empty(shape, dtype=torch.float64, device=cuda)
        plan.c2r([kd], [x_ref])
        x_na = torch.full(shape, float("nan"), dtype=torch.float64, device=cuda)
        dd._lib.call("dd_fft_c2r_noalloc", plan.handle, ctypes.c_void_p(kd.data_ptr()),
                     ctypes.c_void_p(x_na.data_ptr()), st)
        torch.cuda.synchronize()
        a, b = x_na.cpu().numpy(), x_ref.cpu().numpy()
        assert np.isfinite(a).all(), "call %d left unwritten outputs" % call
        assert _rel(a, b) < 1e-13, "call %d" % call
    # the claim itself: a further call takes no device memory
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    dd._lib.call("dd_fft_c2r_noalloc", plan.handle, ctypes.c_void_p(kd.data_ptr()),
                 ctypes.c_void_p(x_na.data_ptr()), st)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


@pytest.mark.gpu
def test_noalloc_rejects_grids_beyond_the_static_buffer(dd, cuda):
    import torch
    shape = (128, 128, 128)  # needs about 19 MB of scratch
    plan = dd.engine.Plan(shape, (2 * np.pi,) * 3)
    kd = torch.zeros(plan.kshape, dtype=torch.complex128, device=cuda)
    xd = torch.zeros(shape, dtype=torch.float64, device=cuda)
    with pytest.raises(NotImplementedError, match="static buffer"):
        dd._lib.call("dd_fft_c2r_noalloc", plan.handle, ctypes.c_void_p(kd.data_ptr()),
                     ctypes.c_void_p(xd.data_ptr()), None)
