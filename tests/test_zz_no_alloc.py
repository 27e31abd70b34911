"""qpc_fieldfree_noalloc: the field-free step for callers that cannot allocate
device memory (a host framework that owns all device allocations through its
own pool, code running during stream capture, a fixed device-memory budget).
The caller owns every buffer; the entry point uses only the scratch array
compiled into the library.  Its results must equal the handle-based entry
point's (qpc_lgwz_propagate_free) and the CPU oracle's on two calls in a row,
for few chains (P lanes per chain) and many (one lane per chain), one m and
several, and it must reject a size beyond its fixed scratch with an error
instead of touching the GPU.

Collected last on purpose, so that a run stopping at the first failure has
already run every other test."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tolerance of the other single-step parity tests


def _problem(q, n_r=96, p=6, n_l=7, B=3, n_m=1, m0=0, seed=21):
    dt = 0.05
    lmax = n_l - 1 + max(abs(m0), abs(m0 + n_m - 1))
    t = q.linear_knots(n_r, p, 0.0, n_r / 2.0)
    S, R, _, _, H = q.radial_setup(n_r, p, lmax + 1, t)
    rng = np.random.default_rng(seed)
    c0 = rng.standard_normal((B, n_m, n_l, n_r)) + 1j * rng.standard_normal((B, n_m, n_l, n_r))
    return dict(n_r=n_r, p=p, n_l=n_l, n_m=n_m, m0=m0, dt=dt, B=B, lmax=lmax, S=S, R=R, H=H, c0=c0)


def _free_device_bytes(torch):
    return torch.cuda.mem_get_info()[0]


def _check(q, oracle, pr, check_alloc=False):
    torch = pytest.importorskip("torch")
    B, n_m, n_l, n_r = pr["B"], pr["n_m"], pr["n_l"], pr["n_r"]
    S, R, H, dt, c0 = pr["S"], pr["R"], pr["H"], pr["dt"], pr["c0"]
    # the existing entry point: two field-free steps through a handle
    prop = q.propagator_cn_hc_lgwz().initialize(n_r, pr["p"], n_l, S, R, H, dt, n_m=n_m, m0=pr["m0"], n_inst=B)
    prop.put(c0)
    prop.propagate()
    ref1 = prop.get()
    prop.propagate()
    ref2 = prop.get()
    prop.close()
    # the CPU oracle of the reference's field-free step (cn_hc_propagate0)
    g = oracle.grid(S, R, H, dt, n_l, n_m=n_m, m0=pr["m0"], n_inst=B)
    o1 = oracle.step(g, c0.reshape(B, -1))
    o2 = oracle.step(g, o1)
    # the no-allocation entry point on buffers this caller owns
    dev = torch.device("cuda:0")
    ff = q.fieldfree_factors(S, H, dt, pr["lmax"])
    S_d = torch.from_numpy(np.ascontiguousarray(S)).to(dev)
    ff_d = torch.from_numpy(np.ascontiguousarray(ff).view(np.float64).copy()).to(dev)
    c_d = torch.from_numpy(np.ascontiguousarray(c0).view(np.float64).copy()).to(dev)
    dims = q.qpc_dims(n_r, pr["p"], n_l, n_m, pr["m0"], B)
    q.fieldfree_noalloc(dims, S_d.data_ptr(), ff_d.data_ptr(), c_d.data_ptr(), 0)
    torch.cuda.synchronize()
    got1 = c_d.cpu().numpy().view(np.complex128).reshape(c0.shape)
    got1_d = c_d.clone()
    unchanged = False
    for _ in range(5):
        # free device memory is a whole-device figure that other processes move too:
        # the second call allocated nothing if one of several tries sees no change
        c_d.copy_(got1_d)
        torch.cuda.synchronize()
        before = _free_device_bytes(torch)
        q.fieldfree_noalloc(dims, S_d.data_ptr(), ff_d.data_ptr(), c_d.data_ptr(), 0)
        torch.cuda.synchronize()
        if _free_device_bytes(torch) == before:
            unchanged = True
            break
    if not unchanged:
        pytest.fail("free device memory changed on each of 5 tries of the second call")
    got2 = c_d.cpu().numpy().view(np.complex128).reshape(c0.shape)
    assert rel_l2(got1, ref1) < TOL
    assert rel_l2(got2, ref2) < TOL
    assert rel_l2(got1.reshape(B, -1), o1) < TOL
    assert rel_l2(got2.reshape(B, -1), o2) < TOL


def test_noalloc_matches_handle_and_oracle_on_two_calls(q, oracle):
    """few chains (3 x 7): P lanes per chain"""
    _check(q, oracle, _problem(q))


def test_noalloc_many_chains(q, oracle):
    """512 x 8 = 4096 chains: one lane per chain"""
    _check(q, oracle, _problem(q, n_r=64, p=6, n_l=8, B=512, seed=5))


def test_noalloc_several_m(q, oracle):
    """n_m = 3, m0 = -1: the factor rows of l = il + |m| up to n_l - 1 + max|m|"""
    _check(q, oracle, _problem(q, n_r=80, p=5, n_l=5, B=2, n_m=3, m0=-1, seed=9))


def test_noalloc_rejects_sizes_beyond_its_scratch(q):
    torch = pytest.importorskip("torch")
    pr = _problem(q)
    dev = torch.device("cuda:0")
    small = torch.zeros(16, dtype=torch.float64, device=dev)
    too_many = q.NOALLOC_MAX_ELEMS // (pr["n_l"] * pr["n_r"]) + 1
    dims = q.qpc_dims(pr["n_r"], pr["p"], pr["n_l"], 1, 0, too_many)
    with pytest.raises(q.QpcError) as e:
        q.fieldfree_noalloc(dims, small.data_ptr(), small.data_ptr(), small.data_ptr(), 0)
    assert e.value.code == 1
    assert "fixed scratch" in str(e.value)
