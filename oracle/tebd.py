"""Restatement of TEBD gate application (test infrastructure only: the product
never imports this module): bond_evolution / bond_evolution3 /
bond_evolution4, _swap_gate, _move! and apply! of circuit/apply_gates.jl:3-187
on numpy tensors.  The state is a list of right-canonical tensors and a list of
L+1 singular-value vectors (0-based: s[i-1] is the reference's s[i]).
Gates are (positions, matrix) pairs over the fused physical index, first site
fastest.
"""

import numpy as np

from .core import stable_tsvd

__all__ = ["bond_evolution", "apply_gate", "apply_circuit", "dense_apply"]


def _split(M, trunc):
    u, s, vh, err = stable_tsvd(M, trunc)
    return s, vh, err


def bond_evolution(G, s1, tensors, trunc):
    """bond_evolution{,3,4} (apply_gates.jl:11-52) for n = len(tensors) sites:
    theta = gate * (A_1 ... A_n); the left s multiplied in; successive cuts,
    each left tensor recovered as (the uncut part) * v^H."""
    Dl = tensors[0].shape[0]
    x = tensors[0]
    for A in tensors[1:]:
        x = np.tensordot(x, A, axes=([x.ndim - 1], [0]))
    dims = [A.shape[1] for A in tensors]
    Dr = tensors[-1].shape[2]
    P = int(np.prod(dims))
    theta = np.einsum("qp,apb->aqb", G, x.reshape(Dl, P, Dr, order="F"))
    cur = theta.reshape(Dl, -1, order="F")
    scaled = s1[:, None] * cur
    outs, svals, err = [], [], 0.0
    left = Dl
    for t in range(len(dims) - 1):
        d = dims[t]
        rest = cur.size // (left * d)
        s, vh, e = _split(scaled.reshape(left * d, rest, order="F"), trunc)
        err = max(err, e)
        k = s.shape[0]
        u = cur.reshape(left * d, rest, order="F") @ vh.conj().T
        outs.append(u.reshape(left, d, k, order="F"))
        svals.append(s)
        cur = vh
        scaled = s[:, None] * vh
        left = k
    outs.append(cur.reshape(left, dims[-1], Dr, order="F"))
    return outs, svals, err


def _swap(s1, A1, A2, trunc):
    d1, d2 = A1.shape[1], A2.shape[1]
    G = np.zeros((d1 * d2, d1 * d2))
    for a in range(d1):
        for b in range(d2):
            G[b + d2 * a, a + d1 * b] = 1.0
    Dl, Dr = A1.shape[0], A2.shape[2]
    x = np.tensordot(A1, A2, axes=([2], [0])).reshape(Dl, d1 * d2, Dr, order="F")
    theta = np.einsum("qp,apb->aqb", G, x).reshape(Dl * d2, d1 * Dr, order="F")
    s, vh, err = _split((s1[:, None] * theta.reshape(Dl, -1, order="F")).reshape(
        Dl * d2, d1 * Dr, order="F"), trunc)
    u = theta @ vh.conj().T
    k = s.shape[0]
    return u.reshape(Dl, d2, k, order="F"), s, vh.reshape(k, d1, Dr, order="F"), err


def _move(mps, s, i, j, trunc):
    err = 0.0
    if i < j:
        for k in range(i, j):
            mps[k - 1], s[k], mps[k], e = _swap(s[k - 1], mps[k - 1], mps[k], trunc)
            err = max(err, e)
    elif i > j:
        for k in range(i, j, -1):
            mps[k - 2], s[k - 1], mps[k - 1], e = _swap(s[k - 2], mps[k - 2], mps[k - 1], trunc)
            err = max(err, e)
    return err


def apply_gate(pos, G, mps, s, trunc):
    """_apply_impl (apply_gates.jl:76-163); 1-based positions, sorted."""
    n = len(pos)
    if n == 1:
        A = mps[pos[0] - 1]
        mps[pos[0] - 1] = np.einsum("qp,apb->aqb", G, A)
        return 0.0
    j = pos[1]
    targets = list(range(j - 1, j - 1 + n))
    err = 0.0
    nn = list(pos) == targets
    order = [(pos[0], j - 1)] + [(pos[t], j - 1 + t) for t in range(2, n)]
    if not nn:
        for a, b in order:
            err = max(err, _move(mps, s, a, b, trunc))
    outs, svals, e = bond_evolution(G, s[j - 2], [mps[t - 1] for t in targets], trunc)
    err = max(err, e)
    for t, A in zip(targets, outs):
        mps[t - 1] = A
    for t, sv in zip(targets[1:], svals):
        s[t - 1] = sv
    if not nn:
        back = [(j - 1, pos[0])] + [(j - 1 + t, pos[t]) for t in range(2, n)]
        if n == 4:
            back = [back[0], back[2], back[1]]
        for a, b in back:
            err = max(err, _move(mps, s, a, b, trunc))
    return err


def apply_circuit(gates, mps, s, trunc):
    return [apply_gate(pos, G, mps, s, trunc) for pos, G in gates]


def dense_apply(psi, L, dims, pos, G):
    """The gate applied to a dense state vector (site 1 fastest)."""
    t = psi.reshape(dims[::-1])                       # axes L..1
    axes = [L - p for p in pos]
    n = len(pos)
    Gt = G.reshape([dims[p - 1] for p in pos][::-1] * 2)       # (out_n..out_1, in_n..in_1)
    ax_in = list(range(n, 2 * n))
    out = np.tensordot(Gt, t, axes=(ax_in, axes[::-1]))
    out = np.moveaxis(out, list(range(n)), axes[::-1])
    return out.reshape(-1)
