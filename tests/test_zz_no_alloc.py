"""qpc_fieldfree_noalloc: the field-free step for callers that cannot allocate
device memory (a host framework that owns all device allocations through its
own pool, code running during stream capture, a fixed device-memory budget).
The caller owns every buffer; the entry point uses only the scratch array
compiled into the library.  Its results must equal the handle-based entry
point's (qpc_lgwz_propagate_free) on two calls in a row, and it must reject a
size beyond its fixed scratch with an error instead of touching the GPU.

Collected last on purpose, so that a run stopping at the first failure has
already run every other test."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tolerance of the other single-step parity tests


def _problem(q):
    n_r, p, n_l, dt, B = 96, 6, 7, 0.05, 3
    t = q.linear_knots(n_r, p, 0.0, 48.0)
    S, R, _, _, H = q.radial_setup(n_r, p, n_l, t)
    rng = np.random.default_rng(21)
    c0 = rng.standard_normal((B, 1, n_l, n_r)) + 1j * rng.standard_normal((B, 1, n_l, n_r))
    return n_r, p, n_l, dt, B, S, R, H, c0


def test_noalloc_matches_handle_on_two_calls(q):
    torch = pytest.importorskip("torch")
    n_r, p, n_l, dt, B, S, R, H, c0 = _problem(q)
    # the existing entry point: two field-free steps through a handle
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, p, n_l, S, R, H, dt, n_inst=B)
    prop.put(c0)
    prop.propagate()
    ref1 = prop.get()
    prop.propagate()
    ref2 = prop.get()
    prop.close()
    # the no-allocation entry point on buffers this caller owns
    dev = torch.device("cuda:0")
    ff = q.fieldfree_factors(S, H, dt, n_l - 1)
    S_d = torch.from_numpy(np.ascontiguousarray(S)).to(dev)
    ff_d = torch.from_numpy(np.ascontiguousarray(ff).view(np.float64).copy()).to(dev)
    c_d = torch.from_numpy(np.ascontiguousarray(c0).view(np.float64).copy()).to(dev)
    dims = q.qpc_dims(n_r, p, n_l, 1, 0, B)
    q.fieldfree_noalloc(dims, S_d.data_ptr(), ff_d.data_ptr(), c_d.data_ptr(), 0)
    torch.cuda.synchronize()
    got1 = c_d.cpu().numpy().view(np.complex128).reshape(B, 1, n_l, n_r)
    free_before = torch.cuda.mem_get_info()[0]
    q.fieldfree_noalloc(dims, S_d.data_ptr(), ff_d.data_ptr(), c_d.data_ptr(), 0)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    got2 = c_d.cpu().numpy().view(np.complex128).reshape(B, 1, n_l, n_r)
    assert rel_l2(got1, ref1) < TOL
    assert rel_l2(got2, ref2) < TOL
    # the second call allocated no device memory
    assert free_after == free_before


def test_noalloc_rejects_sizes_beyond_its_scratch(q):
    torch = pytest.importorskip("torch")
    n_r, p, n_l, dt, B, S, R, H, c0 = _problem(q)
    dev = torch.device("cuda:0")
    small = torch.zeros(16, dtype=torch.float64, device=dev)
    too_many = q.NOALLOC_MAX_ELEMS // (n_l * n_r) + 1
    dims = q.qpc_dims(n_r, p, n_l, 1, 0, too_many)
    with pytest.raises(q.QpcError) as e:
        q.fieldfree_noalloc(dims, small.data_ptr(), small.data_ptr(), small.data_ptr(), 0)
    assert e.value.code == 1
    assert "fixed scratch" in str(e.value)
