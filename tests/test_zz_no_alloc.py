"""The allocation-free interpolation entry point agrees with the allocating one.

``l3es_interp_dft_noalloc`` serves callers that cannot let the library allocate
device memory (for instance a JAX/XLA FFI custom call, where XLA has already
reserved the GPU for its own pool). It keeps its scratch in a fixed array inside
the library, shared by all calls. This file is named so pytest collects it last;
it passes on its own in a fresh process and after the rest of the suite.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 2e-5  # the tolerance of the other GPU parity tests


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _case(dim, n, seed):
    rng = np.random.default_rng(seed)
    shape = (3, n, n, n) if dim == 3 else (3, n, n, 1)
    axes = (1, 2, 3) if dim == 3 else (1, 2)
    u = rng.standard_normal(shape)
    uh = np.fft.rfftn(u, axes=axes).reshape((3, n, n, n // 2 + 1) if dim == 3 else (3, n, n // 2 + 1))
    r = rng.uniform(0.0, 2 * np.pi, size=(700, dim))
    return (torch.from_numpy(np.ascontiguousarray(uh, dtype=np.complex64)).cuda(),
            torch.from_numpy(r).cuda())


def _with_plan(dim, n, c, uh, r):
    from l3es import _native

    p = _native.InterpPlan(dim=dim, ckp_n=c, n_fine=n, np_max=r.shape[0])
    p.set_spectrum(uh)
    out = torch.empty_like(r)
    p.interp(r, out, backend="dft")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice():
    from l3es import _native

    # two calls in a row on the shared scratch: a 3D field at the size limit, then a
    # smaller 2D one (the second must not see anything left by the first)
    for dim, n, c, seed in ((3, 64, 32, 1), (2, 128, 16, 2)):
        uh, r = _case(dim, n, seed)
        got = torch.empty_like(r)
        _native.interp_dft_noalloc(dim, n, c, uh, r, got)
        torch.cuda.synchronize()
        ref = _with_plan(dim, n, c, uh, r)
        assert _rel(got.cpu().numpy(), ref) < RTOL


def test_noalloc_ignores_the_previous_calls_scratch_and_allocates_nothing():
    """A call at the same size right after a call on a different field gives that
    field's answer (stale scratch would show), and a call whose inputs and outputs
    already exist leaves the device's free memory unchanged."""
    from l3es import _native

    uh_a, r = _case(3, 64, 5)
    uh_b, _ = _case(3, 64, 6)
    ref_b = _with_plan(3, 64, 32, uh_b, r)
    got = torch.empty_like(r)
    _native.interp_dft_noalloc(3, 64, 32, uh_a, r, got)  # fills the scratch with field a
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _native.interp_dft_noalloc(3, 64, 32, uh_b, r, got)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert _rel(got.cpu().numpy(), ref_b) < RTOL
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from l3es import _native

    uh, r = _case(3, 128, 3)
    out = torch.empty_like(r)
    with pytest.raises(RuntimeError, match="limit"):
        _native.interp_dft_noalloc(3, 128, 64, uh, r, out)
