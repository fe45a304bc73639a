"""Batches of expansions of different orders: zest_gpu_zt_rotate_backward_ragged
(rotate every expansion, then backward-transform each to its own grid; in
FP64 one rotation launch for all, in split precision the X(+-pi/2) products
of all vectors of one l as split GEMMs; replayed from a CUDA graph on
repeated calls), and the autotuner of the FP64 tile shapes.

The batch must give what per-item zest_gpu_zt_rotate + zest_gpu_zt_backward
give (1e-13 relative max-norm in FP64; 1e-11 in split precision), on the
first (eager) call and on a graph replay with new inputs in the same buffers."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size, zt_grid_shape

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


def rand_zt(rng, L):
    c = np.zeros((zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[zidx(n, l, m)] = rng.normal(size=2) * (n + 1) ** -1.0
                if m == 0:
                    c[zidx(n, l, m), 1] = 0.0
    return c.ravel()


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_batch(rng, orders):
    cs = [rand_zt(rng, int(L)) for L in orders]
    e = np.stack([rng.uniform(0, 2 * np.pi, len(orders)), np.arccos(rng.uniform(-1, 1, len(orders))),
                  rng.uniform(0, 2 * np.pi, len(orders))], axis=1)
    return cs, e


def per_item(ctx, orders, cs, e, rtype):
    rot, grids = [], []
    for L, c, a in zip(orders, cs, e):
        r = ctx.zt_rotate(c.copy(), int(L), a.copy(), rotation_type=rtype)
        rot.append(r)
        grids.append(ctx.zt_backward(r, int(L)))
    return rot, grids


@pytest.mark.parametrize("precision,tol", [(0, 1e-13), (1, 1e-11)])
def test_ragged_batch_matches_per_item(ctx, precision, tol):
    torch = pytest.importorskip("torch")
    import zest_gb300 as zg
    rng = np.random.default_rng(10 + precision)
    orders = np.sort(rng.integers(8, 41, size=40))
    gsz = [int(np.prod(zt_grid_shape(int(L)))) for L in orders]
    coeffs = torch.zeros(sum(2 * zt_coeff_size(int(L)) for L in orders), dtype=torch.float64, device="cuda")
    euler = torch.zeros(3 * len(orders), dtype=torch.float64, device="cuda")
    grids = torch.zeros(sum(gsz), dtype=torch.float64, device="cuda")
    ctx.set_precision(precision)
    try:
        for call in range(2):  # eager + capture, then graph replay with new inputs
            cs, e = make_batch(rng, orders)
            coeffs.copy_(torch.from_numpy(np.concatenate(cs)))
            euler.copy_(torch.from_numpy(e.ravel()))
            ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
            ctx.synchronize()
            ctx.set_precision(zg.PRECISION_FP64)
            rot, want = per_item(ctx, orders, cs, e, 0)
            ctx.set_precision(precision)
            got_c = coeffs.cpu().numpy()
            got_g = grids.cpu().numpy()
            co = go = 0
            for i, L in enumerate(orders):
                n = 2 * zt_coeff_size(int(L))
                # split precision rotates on the tensor cores too (its bound, 1e-11)
                assert relmax(got_c[co:co + n], rot[i]) < (1e-13 if precision == 0 else 1e-11), (call, i)
                assert relmax(got_g[go:go + gsz[i]], want[i]) < tol, (call, i)
                co += n
                go += gsz[i]
    finally:
        ctx.set_precision(0)


@pytest.mark.parametrize("precision", [0, 1])
def test_ragged_graph_recorded_anew_after_buffers_are_freed(ctx, precision):
    # A repeated call replays a CUDA graph that holds the context's scratch,
    # table and work-list pointers.  A transform that regrows the scratch, and
    # trim(), free buffers the graph used: the next call must record a new
    # graph (and give the same results), not replay the old one.
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(40 + precision)
    orders = np.sort(rng.integers(8, 25, size=12))
    gsz = sum(int(np.prod(zt_grid_shape(int(L)))) for L in orders)
    cs, e = make_batch(rng, orders)
    c0 = torch.from_numpy(np.concatenate(cs)).cuda()
    coeffs = torch.empty_like(c0)
    euler = torch.from_numpy(e.ravel()).cuda()
    grids = torch.zeros(gsz, dtype=torch.float64, device="cuda")

    def call():
        coeffs.copy_(c0)
        ctx.zt_rotate_backward_ragged(orders, coeffs, euler, grids)
        ctx.synchronize()
        return coeffs.cpu().numpy(), grids.cpu().numpy()

    ctx.set_precision(precision)
    try:
        ref = call()  # eager run, then the graph is recorded
        runs = [call()]  # replay
        big = np.concatenate([rand_zt(rng, 48) for _ in range(6)])
        ctx.zt_backward(big, 48, batch=6)  # regrows the shared scratch
        runs.append(call())
        ctx.trim()  # frees every buffer
        runs.append(call())
        for i, (c, g) in enumerate(runs):
            assert relmax(c, ref[0]) < 1e-14, i
            assert relmax(g, ref[1]) < 1e-14, i
    finally:
        ctx.set_precision(0)


def test_ragged_rejects_unsorted_orders(ctx):
    torch = pytest.importorskip("torch")
    import zest_gb300 as zg
    c = torch.zeros(2 * (zt_coeff_size(9) + zt_coeff_size(8)), dtype=torch.float64, device="cuda")
    e = torch.zeros(6, dtype=torch.float64, device="cuda")
    g = torch.zeros(int(np.prod(zt_grid_shape(9))) + int(np.prod(zt_grid_shape(8))), dtype=torch.float64,
                    device="cuda")
    with pytest.raises(zg.ZestGPUError) as ex:
        ctx.zt_rotate_backward_ragged([9, 8], c, e, g)
    assert ex.value.code == zg.ERR_INVALID


def test_autotuned_tiles_give_the_same_transforms(ctx):
    import zest_gb300 as zg
    rng = np.random.default_rng(20)
    c2 = zg.Context(0)
    try:
        c2.set_autotune(True)
        for L, batch in [(12, 3), (40, 2), (100, 1)]:
            cs = np.concatenate([rand_zt(rng, L) for _ in range(batch)])
            g_ref = ctx.zt_backward(cs, L, batch=batch)
            g_tuned = c2.zt_backward(cs, L, batch=batch)
            assert relmax(g_tuned, g_ref) < 1e-13
            f_ref = ctx.zt_forward(g_ref, L, batch=batch)
            f_tuned = c2.zt_forward(g_ref, L, batch=batch)
            assert relmax(f_tuned, f_ref) < 1e-13
    finally:
        c2.close()
