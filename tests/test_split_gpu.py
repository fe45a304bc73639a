"""Split-precision form (BF16 fixed-point slices on tcgen05, exact FP32 level
sums, FP64 recombination).

The emulated product is checked first on integer inputs, where it must be
exact, then on random FP64 data against numpy's FP64 product; the Zernike
transforms in split precision are checked against the FP64 path and the
oracle.  Tolerance: 1e-11 relative max-norm (the precision target of the split
form), max|x - x_ref| / max|x_ref|."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size

pytestmark = pytest.mark.gpu

SPLIT_TOL = 1e-11


def relmax(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def ctx():
    import zest_gb300
    from zest_gb300 import build
    build.build()
    c = zest_gb300.Context(0)
    yield c
    c.close()


@pytest.fixture()
def split(ctx):
    import zest_gb300
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    yield ctx
    ctx.set_precision(zest_gb300.PRECISION_FP64)


def rand_zt(rng, L, power=1.5, batch=1):
    c = np.zeros((batch, zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            for m in range(l + 1):
                c[:, zidx(n, l, m)] = rng.normal(size=(batch, 2)) * (n + 1) ** -power
                if m == 0:
                    c[:, zidx(n, l, m), 1] = 0.0
    return c


@pytest.mark.parametrize("M,N,K", [(128, 80, 16), (1, 1, 1), (129, 81, 17), (300, 200, 208), (1000, 37, 256),
                                   (256, 33, 48), (200, 161, 64)])
def test_split_gemm_exact_on_integers(split, M, N, K):
    # integers with |x| < 2^20 are represented exactly by 6 slices of 8 bits
    # (the dropped products involve only zero digits), and the level sums are
    # exact: the product must be exact
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-(1 << 19), 1 << 19, size=(M, K)).astype(np.float64)
    B = rng.integers(-(1 << 19), 1 << 19, size=(N, K)).astype(np.float64)
    C = split.split_gemm(A, B)
    ref = A @ B.T
    # integer products exceed 2^53 only past ~2^40 magnitudes; compare exactly where representable
    assert np.max(np.abs(C - ref) / np.maximum(np.abs(ref), 1.0)) < 1e-15


@pytest.mark.parametrize("S", [4, 5, 6])
def test_split_gemm_random(ctx, S):
    import zest_gb300
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, S)
    try:
        rng = np.random.default_rng(S)
        A = rng.normal(size=(517, 201)) * np.exp(rng.normal(size=(517, 1)))
        B = rng.normal(size=(93, 201))
        C = ctx.split_gemm(A, B)
        err = relmax(C, A @ B.T)
        bound = {4: 1e-7, 5: 1e-9, 6: 5e-12}[S]
        assert err < bound, err
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)


def split_model(A, B, S):
    """Integer model of the split product: balanced base-256 digits of the
    row-scaled operands (rounded to nearest, ties away from zero), levels 0..S-1 summed exactly over K-chunks of at most
    256 terms, each chunk scaled by 2^(eA + eB - 8 (S + 1)) and the chunks
    added in FP64, first to last."""
    K = A.shape[1]
    bits, top = 8, S - 1
    base = 1 << bits

    def digits(X):
        E = np.frexp(np.abs(X).max(axis=1))[1]
        e = E + 1
        y = X * np.exp2(bits * S - e)[:, None]  # exact: a power-of-two scale
        v = (np.sign(y) * np.floor(np.abs(y) + 0.5)).astype(np.int64)  # ties away from zero
        d = np.zeros((S,) + X.shape, dtype=np.int64)
        w = v.copy()
        for s in range(S - 1, 0, -1):
            r = w & (base - 1)
            r = np.where(r >= base // 2, r - base, r)
            d[s] = r
            w = (w - r) >> bits
        d[0] = w
        return d, e
    da, ea = digits(A)
    db, eb = digits(B)
    scale = np.exp2(ea[:, None] + eb[None, :] - bits * (top + 2))
    out = np.zeros((A.shape[0], B.shape[0]))
    for k0 in range(0, K, 256):
        ks = slice(k0, min(K, k0 + 256))
        T = np.zeros((A.shape[0], B.shape[0]), dtype=object)
        for lev in range(top + 1):
            acc = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
            for s in range(S):
                t = lev - s
                if 0 <= t < S:
                    acc += da[s][:, ks] @ db[t][:, ks].T
            T = T * base + acc.astype(object)
        out = out + T.astype(float) * scale
    return out


@pytest.mark.parametrize("K", [1, 16, 33, 64, 208, 256, 257, 400, 992, 2048])
def test_split_gemm_matches_integer_model(split, K):
    # The kernel sums every level in its own FP32 accumulator: levels 0..3
    # exactly, levels 4 and 5 (2^-32 and 2^-40 of level 0) rounded to
    # integers once they pass 2^24.  It must agree with the all-integer model
    # to 1e-13 of the largest entry, with one K-chunk (K <= 256) and with
    # several (257 up to 2048).
    rng = np.random.default_rng(100 + K)
    A = rng.normal(size=(130, K)) * np.exp(rng.normal(size=(130, 1)))
    B = rng.normal(size=(70, K))
    C = split.split_gemm(A, B)
    model = split_model(A, B, 6)
    assert np.max(np.abs(C - model)) <= 1e-13 * np.max(np.abs(model))


@pytest.mark.parametrize("L,batch", [(2, 1), (7, 3), (20, 2), (64, 2)])
def test_split_zt_vs_fp64(ctx, L, batch):
    import zest_gb300
    rng = np.random.default_rng(L)
    c = rand_zt(rng, L, batch=batch).ravel()
    g64 = ctx.zt_backward(c, L, batch=batch)
    f64 = ctx.zt_forward(g64, L, batch=batch)
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        gs = ctx.zt_backward(c, L, batch=batch)
        fs = ctx.zt_forward(g64, L, batch=batch)
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)
    assert relmax(gs, g64) < SPLIT_TOL
    assert relmax(fs, f64) < SPLIT_TOL


@pytest.mark.parametrize("spec", ["dft_f=32,leg_f=32,rad_f=32,rad_b=32,leg_b=80,dft_b=32",
                                  "dft_f=80,leg_f=80,rad_f=80,rad_b=80,leg_b=32,dft_b=80"])
def test_split_zt_column_tiles(ctx, monkeypatch, spec):
    # ZEST_GPU_SPLIT_NT picks each stage's column tile (32: two accumulator
    # sets in TMEM, one MMA per slice of A; 80: one set, MMAs of up to three
    # products) for contexts created after it is set; every choice must give
    # the same split-form results as the FP64 form
    import zest_gb300
    monkeypatch.setenv("ZEST_GPU_SPLIT_NT", spec)
    rng = np.random.default_rng(77)
    L, batch = 57, 3
    c = rand_zt(rng, L, batch=batch).ravel()
    g64 = ctx.zt_backward(c, L, batch=batch)
    f64 = ctx.zt_forward(g64, L, batch=batch)
    c2 = zest_gb300.Context(0)
    try:
        c2.set_precision(zest_gb300.PRECISION_SPLIT, 6)
        gs = c2.zt_backward(c, L, batch=batch)
        fs = c2.zt_forward(g64, L, batch=batch)
    finally:
        c2.close()
    assert relmax(gs, g64) < SPLIT_TOL
    assert relmax(fs, f64) < SPLIT_TOL


@pytest.mark.parametrize("narrow", ["mixed", "64"])
def test_split_zt_narrow_units(ctx, monkeypatch, narrow):
    # ZEST_GPU_SPLIT_NARROW: units of at most 32 valid table rows in a second
    # launch of 32-column tiles ("mixed"), or units of up to 64 rows issued as
    # one MMA per product; the same split-form results as the FP64 form
    import zest_gb300
    monkeypatch.setenv("ZEST_GPU_SPLIT_NARROW", narrow)
    rng = np.random.default_rng(78)
    L, batch = 71, 2
    c = rand_zt(rng, L, batch=batch).ravel()
    g64 = ctx.zt_backward(c, L, batch=batch)
    f64 = ctx.zt_forward(g64, L, batch=batch)
    c2 = zest_gb300.Context(0)
    try:
        c2.set_precision(zest_gb300.PRECISION_SPLIT, 6)
        gs = c2.zt_backward(c, L, batch=batch)
        fs = c2.zt_forward(g64, L, batch=batch)
    finally:
        c2.close()
    assert relmax(gs, g64) < SPLIT_TOL
    assert relmax(fs, f64) < SPLIT_TOL


def test_split_zt_config1_vs_golden(split, golden):
    g = golden("zt_config1")
    c = split.zt_forward(np.ascontiguousarray(g["grid"]).ravel(), 20)
    assert relmax(c, g["coeffs"]) < SPLIT_TOL
    rt = split.zt_backward(np.ascontiguousarray(g["coeffs"]).ravel(), 20)
    assert relmax(rt, g["roundtrip"]) < SPLIT_TOL


def test_split_zt_vs_oracle(split, oracle):
    rng = np.random.default_rng(5)
    L = 33
    c = rand_zt(rng, L)
    g = split.zt_backward(c.ravel(), L)
    assert relmax(g, oracle.zt_backward(c[0], L)) < SPLIT_TOL
    f = split.zt_forward(g, L)
    assert relmax(f, oracle.zt_forward(g, L)) < SPLIT_TOL


@pytest.mark.parametrize("Le,Lg", [(12, 16), (9, 13), (20, 21)])
def test_split_zt_truncation(ctx, Le, Lg):
    # expansions of lower order than the grid (even and odd latitude counts):
    # the spectra of orders m >= Le must enter the inverse DFT as zeros
    import zest_gb300
    rng = np.random.default_rng(9 + Le)
    c = rand_zt(rng, Le).ravel()
    ref_b = ctx.zt_backward(c, Le, Lg)
    g = ctx.zt_backward(c, Le, Le)
    ref_f = ctx.zt_forward(g, Le, Le - 3)
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        assert relmax(ctx.zt_backward(c, Le, Lg), ref_b) < SPLIT_TOL
        assert relmax(ctx.zt_forward(g, Le, Le - 3), ref_f) < SPLIT_TOL
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)


def test_split_zt_full_size_error_budget(ctx):
    # the headline workload's accuracy: order 200, split vs FP64 at 1e-11
    import zest_gb300
    rng = np.random.default_rng(200)
    L, batch = 200, 2
    c = rand_zt(rng, L, batch=batch).ravel()
    g64 = ctx.zt_backward(c, L, batch=batch)
    f64 = ctx.zt_forward(g64, L, batch=batch)
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        gs = ctx.zt_backward(c, L, batch=batch)
        fs = ctx.zt_forward(g64, L, batch=batch)
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)
    for b in range(batch):
        n = g64.size // batch
        assert relmax(gs[b * n:(b + 1) * n], g64[b * n:(b + 1) * n]) < SPLIT_TOL
        k = f64.size // batch
        assert relmax(fs[b * k:(b + 1) * k], f64[b * k:(b + 1) * k]) < SPLIT_TOL


@pytest.mark.parametrize("L", [300, 520])
def test_split_zt_long_sums_in_chunks(ctx, L):
    # orders above 254: the DFT and radial sums (and above 510 the Legendre
    # sums) exceed 256 terms and run as K-chunks; the 1e-11 bound must hold
    import zest_gb300
    rng = np.random.default_rng(L)
    c = rand_zt(rng, L, batch=1).ravel()
    g64 = ctx.zt_backward(c, L)
    f64 = ctx.zt_forward(g64, L)
    ctx.set_precision(zest_gb300.PRECISION_SPLIT, 6)
    try:
        gs = ctx.zt_backward(c, L)
        fs = ctx.zt_forward(g64, L)
    finally:
        ctx.set_precision(zest_gb300.PRECISION_FP64)
    assert relmax(gs, g64) < SPLIT_TOL
    assert relmax(fs, f64) < SPLIT_TOL


@pytest.mark.parametrize("kind,L,batch", [(0, 64, 256), (0, 7, 3), (0, 130, 2), (1, 100, 8), (1, 2, 1), (2, 33, 5),
                                          (2, 34, 4)])
@pytest.mark.parametrize("rtype", [0, 1])
def test_split_single_order_rotation(ctx, kind, L, batch, rtype):
    # Rotor::rotate of a batch of one order in split precision: the two
    # X(+-pi/2) products of every vector as split GEMMs, against the FP64
    # rotation of the same expansions (Zernike, SH and row-skipping spans)
    import zest_gb300 as zg
    rng = np.random.default_rng(1000 * kind + L + 7 * rtype)
    size = {0: zg.zt_coeff_size, 1: zg.st_coeff_size, 2: zg.rows_coeff_size}[kind](L)
    c = rng.normal(size=(batch, size, 2)).ravel()
    e = rng.uniform(-np.pi, np.pi, size=3 * batch)
    fn = {0: ctx.zt_rotate, 1: ctx.st_rotate, 2: ctx.rows_rotate}[kind]
    want = fn(c.copy(), L, e.copy(), batch=batch, rotation_type=rtype)
    ctx.set_precision(zg.PRECISION_SPLIT, 6)
    try:
        got = fn(c.copy(), L, e.copy(), batch=batch, rotation_type=rtype)
    finally:
        ctx.set_precision(zg.PRECISION_FP64)
    for g, w in zip(got.reshape(batch, -1), want.reshape(batch, -1)):
        assert relmax(g, w) < SPLIT_TOL
