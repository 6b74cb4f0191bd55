"""CPU checks of the warm-start network oracle and of the host-side band plan (RCM)."""
import ctypes as C

import numpy as np
import pytest

import mlp_oracle as M


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.140625, 1e-3, 65504.0], np.float32)
    r = M.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties to even -> 1.0
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert r[3] == np.float32(-3.140625)
    # bfloat16 keeps 8 significant bits
    assert abs(r[4] - 1e-3) / 1e-3 < 2 ** -8
    assert r[5] == 65536.0


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = M.init_params(1, out_gain=1.0).astype(np.float64)
    X = rng.standard_normal((20, M.NIN))
    T = rng.standard_normal((20, M.NOUT))
    T[3, 2] = np.nan  # a missing target contributes nothing

    def lossf(q):
        W1, b1, W2, b2, W3, b3 = (q[M.OFF_W1:M.OFF_B1].reshape(M.NIN, M.H), q[M.OFF_B1:M.OFF_W2],
                                  q[M.OFF_W2:M.OFF_B2].reshape(M.H, M.H), q[M.OFF_B2:M.OFF_W3],
                                  q[M.OFF_W3:M.OFF_B3].reshape(M.H, M.NOUT), q[M.OFF_B3:])
        s = lambda z: z / (1 + np.exp(-z))
        y = s(s(X @ W1 + b1) @ W2 + b2) @ W3 + b3
        d = np.where(np.isnan(T), 0.0, y - np.nan_to_num(T))
        return (d * d).sum() / (20 * M.NOUT)

    # float64 parameters, no bfloat16 rounding: the analytic gradient must match central differences
    import mlp_oracle
    orig = mlp_oracle.unpack

    def unpack64(params, bf16=True):
        q = np.asarray(params, np.float64)
        return (q[M.OFF_W1:M.OFF_B1].reshape(M.NIN, M.H), q[M.OFF_B1:M.OFF_W2], q[M.OFF_W2:M.OFF_B2].reshape(M.H, M.H),
                q[M.OFF_B2:M.OFF_W3], q[M.OFF_W3:M.OFF_B3].reshape(M.H, M.NOUT), q[M.OFF_B3:])

    mlp_oracle.unpack = unpack64
    try:
        X32 = X  # forward() casts through float32: use exactly representable inputs
        X[:] = X.astype(np.float32)
        loss, g = M.loss_grad(p, X32, T, bf16=False)
    finally:
        mlp_oracle.unpack = orig
    assert abs(loss - lossf(p)) <= 1e-12 * max(1.0, loss)
    idx = np.random.default_rng(0).choice(M.NPARAMS, 60, replace=False)
    for i in list(idx) + [M.OFF_B3, M.OFF_B1 + 5, M.OFF_W3 + 7]:
        h = 1e-6
        e = np.zeros_like(p)
        e[i] = h
        fd = (lossf(p + e) - lossf(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


def _rcm(eb, n, edges):
    from endobeams_gb300 import _lib
    L = _lib.load()
    adj = [[] for _ in range(n)]
    for a, b in edges:
        adj[a].append(b)
        adj[b].append(a)
    xadj = np.zeros(n + 1, np.int64)
    xadj[1:] = np.cumsum([len(a) for a in adj])
    adjncy = np.array([w for a in adj for w in a], np.int32)
    pos = np.zeros(n, np.int32)
    bw = C.c_int32(0)
    _lib.check(L.eb_rcm_order(n, _lib.ptr(xadj, C.c_int64), _lib.ptr(adjncy, C.c_int32), _lib.ptr(pos, C.c_int32),
                              C.byref(bw)), "eb_rcm_order")
    return pos, bw.value


def test_rcm_path_numbered_from_the_middle(eb):
    """A path whose node 0 sits in the middle: the pseudo-peripheral search needs
    several breadth-first passes before it settles on an end node."""
    n = 101
    order = np.random.default_rng(5).permutation(n)
    order = np.roll(order, -int(np.where(order == 0)[0][0]) + n // 2)  # node 0 in the middle of the path
    edges = [(int(order[i]), int(order[i + 1])) for i in range(n - 1)]
    pos, bw = _rcm(eb, n, edges)
    assert sorted(pos.tolist()) == list(range(n))
    assert bw == 1


def test_rcm_stent_graph_bandwidth(eb, scenes):
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    conf, _, _ = scenes.braided_stent(wires=24, elems_per_wire=60, grid=(2, 2, 2))
    c = conf.beams.conn
    n = len(conf.nodes)
    pos, bw = _rcm(eb, n, [tuple(map(int, e)) for e in c])
    assert sorted(pos.tolist()) == list(range(n))
    assert bw == int(np.abs(pos[c[:, 0]] - pos[c[:, 1]]).max())
    A = sp.coo_matrix((np.ones(len(c)), (c[:, 0], c[:, 1])), shape=(n, n))
    perm = reverse_cuthill_mckee((A + A.T).tocsr(), symmetric_mode=True)
    inv = np.empty(n, int)
    inv[perm] = np.arange(n)
    ref_bw = int(np.abs(inv[c[:, 0]] - inv[c[:, 1]]).max())
    assert bw <= 1.5 * ref_bw + 2
