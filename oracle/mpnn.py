"""Float64 restatement of the learned preconditioner correction (test infrastructure only).

The reference has no counterpart: its linear solves go to a direct or plain Krylov solver
(solvers/nonlinearimplicitstatic.py:547-571, utils/linearsolve.py:35-77).  This module is the
independent implementation the CUDA network (forward, backward, Adam inputs) is checked
against, and it is itself checked against central finite differences in the CPU tests.

Network (per node m of the 3x3-block system, 9 input features):
    a_mn = |K_mn|_F / sum_{n' != m} |K_mn'|_F   (n != m),  a_mm = 0
    h0   = relu(W_in f)
    agg_l = A h_{l-1};  q_l = relu(Ws_l h_{l-1} + Wn_l agg_l);  h_l = h_{l-1} + q_l   (l = 1..3)
    z    = base + so * W_out h3   (0 on masked DOFs)
    loss = 0.5 * scale * sum_free (z - e)^2
Parameter layout: W_in [64][9], then per layer Ws [64][64], Wn [64][64], then W_out [3][64].
"""

import numpy as np
import scipy.sparse as sp

H = 64
FIN = 9
NL = 3
OFF_WIN = 0
OFF_L0 = H * FIN
PER_LAYER = 2 * H * H
OFF_WOUT = OFF_L0 + NL * PER_LAYER
NPARAM = OFF_WOUT + 3 * H


def unpack(P):
    P = np.asarray(P, np.float64)
    W_in = P[OFF_WIN:OFF_L0].reshape(H, FIN)
    layers = []
    for l in range(NL):
        o = OFF_L0 + l * PER_LAYER
        layers.append((P[o : o + H * H].reshape(H, H), P[o + H * H : o + 2 * H * H].reshape(H, H)))
    W_out = P[OFF_WOUT:NPARAM].reshape(3, H)
    return W_in, layers, W_out


def edge_weights(rowPtr, colIdx, vals):
    """Row-normalised Frobenius norms of the off-diagonal blocks (diagonal block -> 0)."""
    rowPtr = np.asarray(rowPtr, np.int64)
    nN = len(rowPtr) - 1
    rows = np.repeat(np.arange(nN), np.diff(rowPtr))
    norms = np.sqrt(np.sum(np.asarray(vals, np.float64).reshape(-1, 9) ** 2, axis=1))
    norms[np.asarray(colIdx) == rows] = 0.0
    tot = np.bincount(rows, weights=norms, minlength=nN)
    inv = np.where(tot > 0, 1.0 / np.where(tot > 0, tot, 1.0), 0.0)
    return norms * inv[rows]


def _adjacency(rowPtr, colIdx, a):
    nN = len(rowPtr) - 1
    return sp.csr_matrix((np.asarray(a, np.float64), np.asarray(colIdx), np.asarray(rowPtr)), shape=(nN, nN))


def forward(rowPtr, colIdx, a, P, f, base, mask, so):
    """Returns z [3 nN] and the activations needed by backward."""
    W_in, layers, W_out = unpack(P)
    A = _adjacency(rowPtr, colIdx, a)
    f = np.asarray(f, np.float64).reshape(-1, FIN)
    h0 = np.maximum(f @ W_in.T, 0.0)
    h = h0
    cache = []
    for Ws, Wn in layers:
        agg = A @ h
        q = np.maximum(h @ Ws.T + agg @ Wn.T, 0.0)
        cache.append((h, agg, q))
        h = h + q
    out = (h @ W_out.T).reshape(-1)
    z = so * out + (0.0 if base is None else np.asarray(base, np.float64))
    if mask is not None:
        z = np.where(np.asarray(mask) != 0, 0.0, z)
    return z, dict(A=A, f=f, h0=h0, cache=cache, h3=h)


def loss_and_grad(rowPtr, colIdx, vals, P, f, base, e, mask, so, scale):
    """(z, loss, dloss/dP) for the network on the graph of `vals`."""
    W_in, layers, W_out = unpack(P)
    a = edge_weights(rowPtr, colIdx, vals)
    z, act = forward(rowPtr, colIdx, a, P, f, base, mask, so)
    d = z - np.asarray(e, np.float64)
    if mask is not None:
        d = np.where(np.asarray(mask) != 0, 0.0, d)
    loss = 0.5 * scale * float(d @ d)
    g = np.zeros(NPARAM)
    dout = (so * scale * d).reshape(-1, 3)
    g[OFF_WOUT:NPARAM] = (dout.T @ act["h3"]).reshape(-1)
    dh = dout @ W_out
    A = act["A"]
    for l in range(NL - 1, -1, -1):
        Ws, Wn = layers[l]
        hprev, agg, q = act["cache"][l]
        du = dh * (q > 0)
        o = OFF_L0 + l * PER_LAYER
        g[o : o + H * H] = (du.T @ hprev).reshape(-1)
        g[o + H * H : o + 2 * H * H] = (du.T @ agg).reshape(-1)
        dh = dh + du @ Ws + A.T @ (du @ Wn)
    du0 = dh * (act["h0"] > 0)
    g[OFF_WIN:OFF_L0] = (du0.T @ act["f"]).reshape(-1)
    return z, loss, g


def random_case(rowPtr, colIdx, seed=0, maskFraction=0.1):
    """Seeded inputs on a given block pattern: symmetric block values, features, base, target,
    mask and weights with a non-zero output layer."""
    rng = np.random.default_rng(seed)
    rowPtr = np.asarray(rowPtr, np.int64)
    colIdx = np.asarray(colIdx, np.int64)
    nN = len(rowPtr) - 1
    rows = np.repeat(np.arange(nN), np.diff(rowPtr))
    # symmetric |K_mn|: value from the unordered pair (m, n)
    lo, hi = np.minimum(rows, colIdx), np.maximum(rows, colIdx)
    key = lo * nN + hi
    uniq, inv = np.unique(key, return_inverse=True)
    base_vals = rng.normal(size=(uniq.size, 9))
    vals = base_vals[inv].astype(np.float32)
    P = np.zeros(NPARAM)
    P[OFF_WIN:OFF_L0] = rng.normal(scale=np.sqrt(2.0 / FIN), size=OFF_L0)
    P[OFF_L0:OFF_WOUT] = rng.normal(scale=0.5 * np.sqrt(1.0 / H), size=OFF_WOUT - OFF_L0)
    P[OFF_WOUT:NPARAM] = rng.normal(scale=np.sqrt(1.0 / H), size=3 * H)
    f = rng.normal(size=(nN, FIN))
    base = rng.normal(size=3 * nN)
    e = rng.normal(size=3 * nN)
    mask = (rng.random(3 * nN) < maskFraction).astype(np.uint8)
    return dict(vals=vals, P=P.astype(np.float32), f=f.astype(np.float32), base=base.astype(np.float32),
                e=e.astype(np.float32), mask=mask)  # fmt: skip


def node_pattern(elements, nNodes):
    """Block pattern (rowPtr, colIdx; sorted rows, diagonal included) of the node graph of a mesh."""
    el = np.asarray(elements, np.int64)
    nn = el.shape[1]
    r = np.repeat(el, nn, axis=1).reshape(-1)
    c = np.tile(el, (1, nn)).reshape(-1)
    key = np.unique(r * nNodes + c)
    rows, cols = key // nNodes, key % nNodes
    rowPtr = np.zeros(nNodes + 1, np.int64)
    np.add.at(rowPtr, rows + 1, 1)
    return np.cumsum(rowPtr).astype(np.int32), cols.astype(np.int32)
