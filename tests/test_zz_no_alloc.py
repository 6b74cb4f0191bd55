"""eb_contact_eval_noalloc: the contact evaluation for callers that cannot
allocate device memory during a call (hosts whose device memory belongs to
their own pool allocator, such as a Julia or PyTorch runtime that has
reserved most of the GPU, and real-time loops that forbid allocation after
start-up).

It reads and writes the caller's device buffers and keeps the prefiltered SDF
coefficients in a fixed device array instead of allocating.  Checked against
the allocating entry point eb_contact_eval on two calls in a row with
different grids and states (the second call must overwrite what the first
left in the shared array), within the discrete-SDF contact tolerance of
test_gpu_element.py.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from states import contact_states, rel_err

pytestmark = pytest.mark.gpu


def _sphere_grid(center, Rs, n, half):
    xs = np.linspace(-half, half, n)
    h = xs[1] - xs[0]
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    field = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - Rs
    surf = np.zeros(14)
    surf[0] = 1
    surf[5:8] = (n, n, n)
    surf[8:11] = center + xs[0]
    surf[11:14] = h
    return field, surf


def _noalloc(eb, inp, props, surf, field):
    import torch

    from endobeams_gb300 import _lib
    L = _lib.load()
    n = inp.shape[0]
    d_in = torch.from_numpy(np.ascontiguousarray(inp)).cuda()
    d_vals = torch.from_numpy(np.ascontiguousarray(field)).cuda()
    d_out = torch.full((n, 301), float("nan"), dtype=torch.float64, device="cuda")
    d_flags = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.eb_contact_eval_noalloc(n, C.c_void_p(d_in.data_ptr()), _lib.ptr(np.ascontiguousarray(eb.GAUSS)),
                                   _lib.ptr(np.ascontiguousarray(props)), _lib.ptr(np.ascontiguousarray(surf)),
                                   C.c_void_p(d_vals.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                   C.c_void_p(d_flags.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    _lib.check(rc, "eb_contact_eval_noalloc")
    return d_out.cpu().numpy(), d_flags.cpu().numpy()


def test_no_alloc_matches_allocating_entry_point(eb):
    cases = [
        (np.array([0.1, -0.2, 0.3]), 1.0, 0.01, np.array([1e4, 0.3, 1e-3, 0.5]), 48, 1.25, 11),
        (np.array([-0.4, 0.0, 0.2]), 0.7, 0.008, np.array([3e3, 0.1, 1e-2, 0.0]), 40, 0.9, 12),
    ]
    for center, Rs, rb, props, n, half, seed in cases:  # two calls in a row
        field, surf = _sphere_grid(center, Rs, n, half)
        inp = contact_states(256, center, Rs, rb, seed=seed)
        ref, ref_flags = eb.contact_eval(inp, props, surf, values=field)
        out, flags = _noalloc(eb, inp, props, surf, field)
        assert np.array_equal(flags, ref_flags)
        touched = ref_flags.astype(bool)
        assert touched.sum() > 100
        assert np.all(out[~touched] == 0.0)  # both paths leave zero records for untouched elements
        for name, a, b, tol in [("E", 0, 1, 1e-9), ("Tc", 1, 13, 1e-10), ("K", 13, 157, 1e-10),
                                ("C", 157, 301, 1e-10)]:
            err = rel_err(out[touched, a:b], ref[touched, a:b])
            assert err.max() <= tol, f"{name}: {err.max():.3e}"


def test_no_alloc_analytic_sphere_and_plane(eb):
    """The analytic surfaces need no SDF array: sphere and plane (the plane reads surf[1] as its
    axis) give the allocating entry point's records, bit for bit (same kernel, same inputs)."""
    from states import plane_states
    props = np.array([1e4, 0.3, 1e-3, 0.5])
    center, Rs, rb = np.array([0.1, -0.2, 0.3]), 1.0, 0.01
    sphere = np.zeros(14)
    sphere[0], sphere[1:4], sphere[4] = 0, center, Rs
    plane = np.zeros(14)
    plane[0], plane[1], plane[2] = 2, 1, 0.013
    for surf, inp in [(sphere, contact_states(256, center, Rs, rb, seed=31)),
                      (plane, plane_states(256, 1, 0.013, rb, seed=32))]:
        ref, ref_flags = eb.contact_eval(inp, props, surf)
        out, flags = _noalloc(eb, inp, props, surf, np.zeros(1))
        assert np.array_equal(flags, ref_flags)
        assert ref_flags.sum() > 100
        assert np.array_equal(out, ref)


def test_no_alloc_rejects_grid_above_limit(eb):
    import torch

    from endobeams_gb300 import _lib
    L = _lib.load()
    n = 70  # 72^3 padded coefficients > 287496
    surf = np.zeros(14)
    surf[0] = 1
    surf[5:8] = (n, n, n)
    surf[11:14] = 0.1
    d = torch.zeros(301, dtype=torch.float64, device="cuda")
    rc = L.eb_contact_eval_noalloc(1, C.c_void_p(d.data_ptr()), _lib.ptr(np.ascontiguousarray(eb.GAUSS)),
                                   _lib.ptr(np.zeros(4)), _lib.ptr(surf), C.c_void_p(d.data_ptr()),
                                   C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert rc == -1
    assert b"EB_NOALLOC_SDF_MAX_COEFS" in L.eb_last_error()


@pytest.mark.parametrize("dims", [(2.0 ** 21 + 3, 2.0 ** 21 + 3, 2.0 ** 21 + 3), (float("nan"), 4, 4),
                                  (float("inf"), 4, 4), (4.5, 4, 4), (0, 4, 4), (-3, 4, 4), (1e30, 1, 1)])
def test_no_alloc_rejects_bad_dimensions_before_launching(eb, dims):
    """Dimensions whose padded product would overflow, non-finite or fractional dimensions are
    rejected on the host: the output buffer keeps its sentinel, so nothing was launched."""
    import torch

    from endobeams_gb300 import _lib
    L = _lib.load()
    surf = np.zeros(14)
    surf[0] = 1
    surf[5:8] = dims
    surf[11:14] = 0.1
    d = torch.full((301,), 7.0, dtype=torch.float64, device="cuda")
    fl = torch.full((1,), 9, dtype=torch.int32, device="cuda")
    rc = L.eb_contact_eval_noalloc(1, C.c_void_p(d.data_ptr()), _lib.ptr(np.ascontiguousarray(eb.GAUSS)),
                                   _lib.ptr(np.zeros(4)), _lib.ptr(surf), C.c_void_p(d.data_ptr()),
                                   C.c_void_p(d.data_ptr()), C.c_void_p(fl.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == -1
    assert b"eb_contact_eval_noalloc" in L.eb_last_error()
    assert torch.all(d == 7.0) and int(fl[0]) == 9
