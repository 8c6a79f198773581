"""The learned search order: tensor-core MLP forward, hand-written backward and
Adam against a NumPy FP64 reference of the same BF16 arithmetic, and the order's
only effect being the search order."""
import numpy as np
import pytest

import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu


def ref_forward(p, X):
    """FP64 reference of the kernels' arithmetic: BF16 inputs, weights and hidden
    activations, FP32-exact sums."""
    Xb = G.bf16_round(X).astype(np.float64)
    W1 = G.bf16_round(p[:8192]).reshape(128, 64).astype(np.float64)
    b1 = p[8192:8320].astype(np.float64)
    W2 = G.bf16_round(p[8320:24704]).reshape(128, 128).astype(np.float64)
    b2 = p[24704:24832].astype(np.float64)
    w3 = G.bf16_round(p[24832:24960]).astype(np.float64)
    b3 = float(p[24960])
    h1 = G.bf16_round(np.maximum(Xb @ W1.T + b1, 0).astype(np.float32)).astype(np.float64)
    h2 = G.bf16_round(np.maximum(h1 @ W2.T + b2, 0).astype(np.float32)).astype(np.float64)
    y = h2 @ w3 + b3
    return Xb, W2, w3, h1, h2, y


def ref_grad(p, X, t):
    Xb, W2, w3, h1, h2, y = ref_forward(p, X)
    n = len(t)
    dy = (1 / (1 + np.exp(-y)) - t) / n
    dh2 = np.outer(dy, w3) * (h2 > 0)
    dh2b = G.bf16_round(dh2.astype(np.float32)).astype(np.float64)
    dh1 = (dh2b @ W2) * (h1 > 0)
    g = np.zeros(G.MLP_PARAMS)
    g[:8192] = (dh1.T @ Xb).ravel()
    g[8192:8320] = dh1.sum(0)
    g[8320:24704] = (dh2.T @ h1).ravel()
    g[24704:24832] = dh2.sum(0)
    g[24832:24960] = dy @ h2
    g[24960] = dy.sum()
    loss = np.mean(np.maximum(y, 0) - y * t + np.log1p(np.exp(-np.abs(y))))
    return g, loss, y


def to_device(ctx, a):
    d = ctx.alloc(a.nbytes)
    ctx.h2d(d, a)
    return d


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(3)
    n = 1000
    X = rng.random((n, 64)).astype(np.float32)
    t = (X[:, 0] + 0.5 * X[:, 5] > 0.8).astype(np.float32)
    return X, t


def test_forward_matches_reference(ctx, data):
    X, _ = data
    p = G.init_mlp_params(11)
    p[8192:8320] = 0.05
    dx = to_device(ctx, G.to_bf16_bits(X))
    dy = ctx.alloc(4 * len(X))
    try:
        ctx.mlp_forward(len(X), dx, p, dy)
        y = ctx.d2h(np.zeros(len(X), np.float32), dy)
    finally:
        ctx.free(dx)
        ctx.free(dy)
    _, _, _, _, _, yr = ref_forward(p, X)
    assert np.allclose(y, yr, rtol=2e-2, atol=2e-2), np.abs(y - yr).max()


def test_gradients_match_reference(ctx, data):
    X, t = data
    p = G.init_mlp_params(12)
    dx = to_device(ctx, G.to_bf16_bits(X))
    dt = to_device(ctx, t)
    try:
        g, loss = ctx.mlp_grad(len(X), dx, dt, p)
    finally:
        ctx.free(dx)
        ctx.free(dt)
    gr, lr, _ = ref_grad(p, X, t)
    assert abs(loss - lr) < 1e-2 * max(1.0, abs(lr))
    # tolerance: BF16 hidden activations and the BF16 dH2 operand of the dH1 product
    for lo, hi in [(0, 8192), (8192, 8320), (8320, 24704), (24704, 24832), (24832, 24960), (24960, 24961)]:
        a, b = g[lo:hi], gr[lo:hi]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-6, (lo, np.linalg.norm(a - b),
                                                                          np.linalg.norm(b))


def test_training_lowers_the_loss(ctx, data):
    X, t = data
    p = G.init_mlp_params(13)
    dx = to_device(ctx, G.to_bf16_bits(X))
    dt = to_device(ctx, t)
    try:
        p2, losses = ctx.mlp_train(len(X), dx, dt, p, epochs=60, batch=256, lr=3e-3)
        dy = ctx.alloc(4 * len(X))
        ctx.mlp_forward(len(X), dx, p2, dy)
        y = ctx.d2h(np.zeros(len(X), np.float32), dy)
        ctx.free(dy)
    finally:
        ctx.free(dx)
        ctx.free(dt)
    assert losses[-1] < 0.6 * losses[0]
    assert ((y > 0) == (t > 0.5)).mean() > 0.9


def test_learned_order_changes_only_the_search_order(ctx):
    n = 512
    d_rows = ctx.alloc(n * 15 * 8)
    outs = []
    try:
        ctx.generate_sts_device(n, 15, 99, True, d_rows)
        for params in (None, G.init_mlp_params(14)):
            ctx.set_ordering(params)
            bufs = [ctx.alloc(n), ctx.alloc(16 * n), ctx.alloc(16 * n), ctx.alloc(n)]
            ctx.check_bibd_device(n, 15, 35, G.COMPLETE | G.RAW | G.AUT_CANON, d_rows, *bufs)
            ctx.stream_sync()
            outs.append([ctx.d2h(np.zeros(n * k, dt), b) for b, k, dt in
                         zip(bufs, (1, 16, 2, 1), (np.uint8, np.uint8, np.uint64, np.uint8))])
            for b in bufs:
                ctx.free(b)
    finally:
        ctx.set_ordering(None)
        ctx.free(d_rows)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


def test_first_row_labels_start_a_canonical_labeling(ctx):
    n = 64
    d_rows = ctx.alloc(n * 15 * 8)
    d_lab = ctx.alloc(2 * n)
    try:
        ctx.generate_sts_device(n, 15, 7, False, d_rows)
        ctx.label_first_rows(n, 15, 35, G.RAW, d_rows, d_lab)
        rows = ctx.d2h(np.zeros(n * 15, np.uint64), d_rows).reshape(n, 15)
        lab = ctx.d2h(np.zeros(n, np.uint16), d_lab)
    finally:
        ctx.free(d_rows)
        ctx.free(d_lab)
    for i in range(24):
        M = oracle.rows_to_matrix(rows[i], 35)
        _, aut, _ = oracle.bibd_canonize(M)
        k = bin(int(lab[i])).count("1")
        # the first rows of the labelings reaching the canonical form are one orbit of
        # Aut(M) on the rows: at least one row, and their number divides |Aut|
        assert k >= 1 and aut % k == 0, (i, k, aut)


def test_config4_eval_batch_learned_order_matches_oracle():
    """Config 4's evaluation batch at full size (1,048,576 fresh STS(15), the bench's
    seed + 1) under a trained learned order: every output equals the plain order's
    on every item, and every 512th item equals the oracle."""
    n, V, B, seed = 1 << 20, 15, 35, 20241203
    ctx = G.Context(max_items=16, aut_cap=1)
    try:
        # a short training run on the training seed's batch (labels from the exact search)
        n_train = 1 << 14
        d_tr = ctx.alloc(n_train * V * 8)
        ctx.generate_sts_device(n_train, V, seed, True, d_tr)
        d_lab = ctx.alloc(2 * n_train)
        ctx.label_first_rows(n_train, V, B, G.RAW, d_tr, d_lab)
        lab = ctx.d2h(np.zeros(n_train, np.uint16), d_lab)
        labels = ((lab[:, None] >> np.arange(V, dtype=np.uint16)) & 1).astype(np.float32).reshape(-1)
        d_feat = ctx.alloc(n_train * V * 64 * 2)
        ctx.mlp_features(n_train, V, B, d_tr, d_feat)
        d_y = to_device(ctx, labels)
        params, _ = ctx.mlp_train(n_train * V, d_feat, d_y, G.init_mlp_params(seed), epochs=1, batch=8192, lr=1e-3)
        for p_ in (d_tr, d_lab, d_feat, d_y):
            ctx.free(p_)
        d_rows = ctx.alloc(n * V * 8)
        ctx.generate_sts_device(n, V, seed + 1, True, d_rows)
        ctx.stream_sync()
        rows = ctx.d2h(np.zeros(n * V, np.uint64), d_rows).reshape(n, V)
        flags = G.COMPLETE | G.RAW | G.AUT_CANON
        outs = {}
        for name, prm in (("plain", None), ("learned", params)):
            ctx.set_ordering(prm)
            d = [ctx.alloc(n), ctx.alloc(16 * n), ctx.alloc(16 * n), ctx.alloc(n)]
            ctx.check_bibd_device(n, V, B, flags, d_rows, *d)
            ctx.stream_sync()
            outs[name] = [ctx.d2h(np.zeros(n * k, np.uint8), p_) for p_, k in zip(d, (1, 16, 16, 1))]
            for p_ in d:
                ctx.free(p_)
        ctx.set_ordering(None)
        ctx.free(d_rows)
    finally:
        ctx.close()
    for a, b in zip(outs["plain"], outs["learned"]):
        assert np.array_equal(a, b)
    can, wit, aut, st = outs["learned"]
    assert not st.any()
    import cases
    cases.compare_sts_sample(rows, can, wit.reshape(n, 16), aut.view(np.uint64).reshape(n, 2), range(0, n, 512))


def test_tensor_core_forward_matches_the_warp_mma_path(data):
    """The forward pass on tcgen05 (X by TMA, FP32 accumulators in tensor memory, 128
    rows per CTA) against the warp-level mma.sync path on the same BF16 inputs: logits
    within BF16 rounding of the hidden layers, on sizes that end inside a 128-row tile
    (batches under 128 rows take the warp-level path in both contexts); and the
    training gradients of both paths agree."""
    X, t = data
    XL = np.random.default_rng(22).random((4095, 64)).astype(np.float32)
    p = G.init_mlp_params(21)
    p[8192:8320] = 0.05
    tc = G.Context(max_items=1 << 12, aut_cap=4)
    mm = G.Context(max_items=1 << 12, aut_cap=4, options=G.OPT_MLP_WARP_MMA)
    try:
        for n in (1, 127, 128, 129, 1000, 4095):
            assert n <= len(XL)
            ys = []
            for c in (tc, mm):
                dx = to_device(c, G.to_bf16_bits(XL[:n]))
                dy = c.alloc(4 * n)
                try:
                    c.mlp_forward(n, dx, p, dy)
                    ys.append(c.d2h(np.zeros(n, np.float32), dy))
                finally:
                    c.free(dx)
                    c.free(dy)
            d = np.abs(ys[0] - ys[1])
            assert d.max() < 2e-2 and np.median(d) < 1e-3, (n, d.max(), np.median(d))
            _, _, _, _, _, yr = ref_forward(p, XL[:n])
            assert np.allclose(ys[0], yr, rtol=2e-2, atol=2e-2), n
        gs = []
        for c in (tc, mm):
            dx = to_device(c, G.to_bf16_bits(X))
            dt = to_device(c, t)
            try:
                gs.append(c.mlp_grad(len(X), dx, dt, p))
            finally:
                c.free(dx)
                c.free(dt)
        (g0, l0), (g1, l1) = gs
        assert abs(l0 - l1) < 1e-3
        assert np.abs(g0 - g1).max() < 5e-3 * max(1.0, np.abs(g1).max())
    finally:
        tc.close()
        mm.close()
