"""CPU reference of the learned line preconditioner -- TEST INFRASTRUCTURE ONLY.

The reference CATHY has no learned component: this module restates, in
numpy, the network and training objective that the CUDA kernels in
pycathy_wrapper_gb300/csrc/learned.cu implement, so that their forward
values and gradients can be checked on the CPU.  Only tests/ import it.

Model (one graph per ensemble member; nodes = mesh nodes, edges = the
off-diagonal slots of the full CSR pattern of the Picard matrix A):

  features  f_s (16, 8 used) of slot s = (i, j):
              a_ij / sqrt(a_ii a_jj), rowsum_i / a_ii, rowsum_j / a_jj,
              scaled log10 Ks_i, scaled log10 dtheta/dh_i, scaled log10 dt,
              vertical flag, scaled log10 (Ks_j / Ks_i)
  layer 1   H1 = bf16(relu(bf16(F) W1b^T + b1))                  (16 -> 64)
  message   M_i = mean of H1 over the off-diagonal slots of row i
  layer 2   U = bf16(H1 + M_row + M_col);  Z2 = U W2b^T + b2;  H2 = relu(Z2)
  layer 3   o = H2 . w3 + b3;  omega = tanh(o) in (-1, 1)
  output    d'_i = a_ii + sum over non-vertical slots s of row i with a
            non-Dirichlet column of omega_s a_ij
            (a learned, per-edge signed version of the row-sum
            compensation of modified incomplete factorisations)

The preconditioner is the column-line block Jacobi factor built on the
corrected diagonal d' and the vertical couplings of A: T' y = r is one
tridiagonal solve per vertical column of the extruded mesh.  omega = 0 is
the plain column-line preconditioner.

Training objective on Krylov pairs (p_k, q_k = A p_k) taken from the plain
solver's own PCG iterations:
  L = mean_k  (T'^-1 q_k - p_k)^T A (T'^-1 q_k - p_k) / (p_k^T q_k)
i.e. the A-norm of the error of the preconditioned map on the directions
the solver actually explores.  With y = T'^-1 q, u = dL/dy = 2 A delta /
den and g = T'^-1 u, dL/dd'_i = -sum_k g_k[i] y_k[i].
"""
from __future__ import annotations

import numpy as np

NF = 16       # padded feature width (the tensor-core K of layer 1)
HID = 64      # hidden width


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), kept as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    out = ((b + r) & 0xFFFF0000).astype(np.uint32)
    return out.view(np.float32).reshape(x.shape)


def init_params(seed=0):
    """Seeded initial parameters (the same recipe as the CUDA initialiser is
    not required: tests pass explicit parameters to both sides)."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((HID, NF), np.float32)
    W1[:, :8] = rng.standard_normal((HID, 8)) * np.sqrt(2.0 / 8)
    W2 = (rng.standard_normal((HID, HID)) * np.sqrt(2.0 / HID)).astype(np.float32)
    w3 = (rng.standard_normal(HID) * 0.1 / np.sqrt(HID)).astype(np.float32)
    return dict(W1=W1, b1=np.zeros(HID, np.float32), W2=W2,
                b2=np.zeros(HID, np.float32), w3=w3,
                b3=np.array([0.0], np.float32))


PARAM_ORDER = ("W1", "b1", "W2", "b2", "w3", "b3")


def pack(params):
    return np.concatenate([np.asarray(params[k], np.float32).ravel() for k in PARAM_ORDER])


def unpack(vec):
    shapes = dict(W1=(HID, NF), b1=(HID,), W2=(HID, HID), b2=(HID,), w3=(HID,), b3=(1,))
    out, o = {}, 0
    for k in PARAM_ORDER:
        sz = int(np.prod(shapes[k]))
        out[k] = np.asarray(vec[o:o + sz], np.float32).reshape(shapes[k])
        o += sz
    return out


class Graph:
    """One member's Picard system in full CSR (0-based) with its nodal data."""

    def __init__(self, rowptr, cols, vals, dmask, nnod, ks, cap, dt):
        self.rowptr = np.asarray(rowptr, np.int64)
        self.cols = np.asarray(cols, np.int64)
        self.vals = np.asarray(vals, np.float64)
        self.dm = np.asarray(dmask, bool)
        self.nnod = int(nnod)
        self.ks = np.asarray(ks, np.float64)
        self.cap = np.asarray(cap, np.float64)
        self.dt = float(dt)
        n = self.n = len(self.rowptr) - 1
        self.rows = np.repeat(np.arange(n), np.diff(self.rowptr))
        self.isdiag = self.rows == self.cols
        self.diag = np.zeros(n)
        self.diag[self.rows[self.isdiag]] = self.vals[self.isdiag]
        self.off = ~self.isdiag
        self.vert = np.abs(self.cols - self.rows) == self.nnod
        # vertical coupling to the node below (i + nnod), masked at Dirichlet
        self.cdown = np.zeros(n)
        sel = (self.cols - self.rows == self.nnod)
        ok = sel & ~self.dm[self.rows] & ~self.dm[self.cols]
        self.cdown[self.rows[ok]] = self.vals[ok]

    # ---- operator with Dirichlet rows as identity (the solver's SpMV) ----
    def matvec(self, x):
        y = np.zeros(self.n)
        np.add.at(y, self.rows, self.vals * x[self.cols])
        y[self.dm] = x[self.dm]
        return y


def features(g: Graph):
    """Edge features (E_off x NF, float32) of the off-diagonal slots."""
    v, rows, cols = g.vals, g.rows, g.cols
    colok = ~g.dm[cols]
    rs = np.zeros(g.n)
    np.add.at(rs, rows, np.where(colok, v, 0.0))
    with np.errstate(divide="ignore", invalid="ignore"):
        rsr = np.where(g.dm, 1.0, rs / g.diag)
    o = g.off
    i, j = rows[o], cols[o]
    d = np.abs(g.diag)
    F = np.zeros((int(o.sum()), NF), np.float64)
    coup = v[o] / np.sqrt(d[i] * d[j])
    coup[g.dm[i] | g.dm[j]] = 0.0
    lk = np.log10(g.ks)
    F[:, 0] = coup
    F[:, 1] = rsr[i]
    F[:, 2] = rsr[j]
    F[:, 3] = (lk[i] + 5.0) * 0.5
    F[:, 4] = np.log10(g.cap[i] + 1e-7) / 3.0 + 1.0
    F[:, 5] = np.log10(g.dt) * 0.5 - 1.0
    F[:, 6] = g.vert[o].astype(np.float64)
    F[:, 7] = (lk[j] - lk[i]) * 0.5
    return F.astype(np.float32)


def forward(g: Graph, P, emulate_bf16=True):
    """Network forward.  Returns a dict with every intermediate."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float32))
    F = r(features(g))
    W1b, W2b = r(P["W1"]), r(P["W2"])
    o_mask = g.off
    i = g.rows[o_mask]
    j = g.cols[o_mask]
    Z1 = F.astype(np.float64) @ W1b.T.astype(np.float64) + P["b1"]
    H1 = r(np.maximum(Z1, 0.0).astype(np.float32)).astype(np.float64)
    deg = np.bincount(i, minlength=g.n).astype(np.float64)
    M = np.zeros((g.n, HID))
    np.add.at(M, i, H1)
    M = (M / np.maximum(deg, 1.0)[:, None]).astype(np.float32)
    H1f = H1.astype(np.float32)
    U = r((H1f + M[i]) + M[j]).astype(np.float64)
    M = M.astype(np.float64)
    Z2 = U @ W2b.T.astype(np.float64) + P["b2"]
    H2 = np.maximum(Z2, 0.0)
    o = H2 @ P["w3"].astype(np.float64) + float(P["b3"][0])
    om = np.tanh(o)
    use = (~g.vert[o_mask]) & (~g.dm[j]) & (~g.dm[i])
    comp = np.zeros(g.n)
    np.add.at(comp, i, np.where(use, om * g.vals[o_mask], 0.0))
    dprime = np.where(g.dm, 1.0, g.diag + comp)
    return dict(F=F, Z1=Z1, H1=H1, M=M, U=U, Z2=Z2, H2=H2, o=o, om=om, use=use,
                dprime=dprime, i=i, j=j, deg=deg, W1b=W1b, W2b=W2b)


# ---- column-line preconditioner ------------------------------------------
def line_factor(g: Graph, dprime):
    """Pivots of the tridiagonal solve along every vertical column."""
    n, nnod = g.n, g.nnod
    nl = n // nnod
    piv = np.zeros(n)
    for c in range(nnod):
        pp, cp = 1.0, 0.0
        for k in range(nl):
            i = c + k * nnod
            a = 1.0 if g.dm[i] else dprime[i]
            p = a - cp * cp / pp
            piv[i] = p
            pp = p
            cp = g.cdown[i] if k + 1 < nl else 0.0
    return piv


def line_solve(g: Graph, piv, r):
    n, nnod = g.n, g.nnod
    nl = n // nnod
    z = np.zeros(n)
    for c in range(nnod):
        idx = c + nnod * np.arange(nl)
        y = np.zeros(nl)
        for k in range(nl):
            i = idx[k]
            y[k] = r[i] - (g.cdown[i - nnod] * y[k - 1] / piv[i - nnod] if k > 0 else 0.0)
        zn = 0.0
        for k in range(nl - 1, -1, -1):
            i = idx[k]
            zk = (y[k] - g.cdown[i] * zn) / piv[i]
            z[i] = zk
            zn = zk
    return z


def loss_and_dd(g: Graph, dprime, pairs):
    """Training loss and its gradient with respect to d'."""
    piv = line_factor(g, dprime)
    L, dd = 0.0, np.zeros(g.n)
    K = 0
    for p, q in pairs:
        den = float(p @ q)
        if den <= 0.0:
            continue
        K += 1
    for p, q in pairs:
        den = float(p @ q)
        if den <= 0.0:
            continue
        y = line_solve(g, piv, q)
        delta = y - p
        Ad = g.matvec(delta)
        L += float(delta @ Ad) / den / K
        u = 2.0 * Ad / den / K
        gg = line_solve(g, piv, u)
        dd -= gg * y
    dd[g.dm] = 0.0
    return L, dd


def backward(g: Graph, P, fw, dd):
    """Parameter gradients given dL/dd' (mirrors the CUDA backward)."""
    i, j = fw["i"], fw["j"]
    vals_off = g.vals[g.off]
    dom = np.where(fw["use"], dd[i] * vals_off, 0.0)
    do = dom * (1.0 - fw["om"] ** 2)
    gw3 = fw["H2"].T @ do
    gb3 = np.array([do.sum()])
    dZ2 = (do[:, None] * P["w3"][None, :].astype(np.float64)) * (fw["Z2"] > 0)
    dZ2b = bf16(dZ2.astype(np.float32)).astype(np.float64)
    gW2 = dZ2b.T @ fw["U"]
    gb2 = dZ2b.sum(axis=0)
    dU = (dZ2b @ fw["W2b"].astype(np.float64)).astype(np.float32).astype(np.float64)
    D = np.zeros((g.n, HID))
    np.add.at(D, i, dU)
    np.add.at(D, j, dU)
    dH1 = dU + D[i] / np.maximum(fw["deg"][i], 1.0)[:, None]
    dZ1 = dH1 * (fw["Z1"] > 0)
    dZ1b = bf16(dZ1.astype(np.float32)).astype(np.float64)
    gW1 = dZ1b.T @ fw["F"].astype(np.float64)
    gb1 = dZ1b.sum(axis=0)
    return dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, w3=gw3, b3=gb3)


def loss_grad(g: Graph, P, pairs, emulate_bf16=True):
    fw = forward(g, P, emulate_bf16)
    L, dd = loss_and_dd(g, fw["dprime"], pairs)
    return L, backward(g, P, fw, dd), fw, dd


def adam(P, G, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step on float32 master parameters (in place)."""
    state["t"] = state.get("t", 0) + 1
    t = state["t"]
    for k in PARAM_ORDER:
        m = state.setdefault("m_" + k, np.zeros_like(P[k], np.float64))
        v = state.setdefault("v_" + k, np.zeros_like(P[k], np.float64))
        m[...] = b1 * m + (1 - b1) * G[k]
        v[...] = b2 * v + (1 - b2) * G[k] ** 2
        mh = m / (1 - b1 ** t)
        vh = v / (1 - b2 ** t)
        P[k] = (P[k] - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32)
    return P
