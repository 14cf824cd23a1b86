"""U(1) block-sparse restatement of the reference's symmetric path (test
infrastructure only: the product never imports this module).

The reference runs DMRG2 on TensorKit tensors whose legs are U1Space
(utilities/models.jl:47 ``heisenberg_xxz_chain``; the charges of
``abelian_matrix_from_dense``, auxiliary/abelianmatrix.jl:112-124: basis
state i of the physical leg has charge i).  TensorKit stores one dense block
per allowed charge combination, contracts block by block, and in ``tsvd!``
factorises each charge sector of the bond separately, then truncates across
sectors (truncation.jl:27-47: cutoff relative to the total norm first, then
keep the D largest values).  TensorKit itself is not vendored in the
reference tree; this module restates that published behaviour:

- a leg is a list of (charge, dim), charges increasing, basis charge-sorted;
- tensors are held dense in the charge-sorted basis with exact zeros outside
  the allowed blocks, so the dense contractions of oracle.core give exactly
  the block-sparse result; ``ac2_prime_blocks`` is the explicit per-block
  loop (the CPU block-sparse baseline);
- ``u1_split`` is the per-sector SVD with the cross-sector truncation.

Ties between equal singular values of different sectors are broken towards
the lower charge (TensorKit's choice is an implementation detail of its
sector iteration order).
"""

import numpy as np

from .core import ac2_prime, simple_lanczos_solver
from .algorithms import OracleEnv

__all__ = ["Leg", "allowed3", "allowed_env", "pack2", "unpack2", "ac2_prime_blocks",
           "u1_split", "U1OracleEnv", "u1_dmrg2_sweep", "channel_charges", "random_u1_state",
           "sector_counts"]


class Leg:
    """A U1Space: sorted (charge, dim) sectors and their basis offsets."""

    def __init__(self, sectors):
        items = sorted((int(q), int(d)) for q, d in (sectors.items() if isinstance(sectors, dict)
                                                     else sectors) if int(d) > 0)
        self.charges = [q for q, _ in items]
        self.dims = [d for _, d in items]
        self.offsets = list(np.cumsum([0] + self.dims[:-1]))
        self.dim = int(sum(self.dims))

    def find(self, q):
        try:
            return self.charges.index(q)
        except ValueError:
            return -1

    def basis_charges(self):
        return np.repeat(np.asarray(self.charges), self.dims)

    def items(self):
        return list(zip(self.charges, self.dims))


def sector_counts(n, qphys):
    c = {0: 1}
    for _ in range(n):
        nxt = {}
        for q, k in c.items():
            for p in qphys:
                nxt[q + p] = nxt.get(q + p, 0) + k
        c = nxt
    return c


def channel_charges(Ws, qphys):
    """MPO bond channel charges: qw(wr) = qw(wl) + qp(s') - qp(s) on every
    nonzero W[wl, s', wr, s], from channel 0 of the left boundary (charge 0),
    propagated in both directions."""
    L = len(Ws)
    q = [[None] * Ws[0].shape[0]] + [[None] * W.shape[2] for W in Ws]
    q[0][0] = 0
    changed = True
    while changed:
        changed = False
        for i, W in enumerate(Ws):
            for wl, so, wr, si in np.argwhere(np.abs(W) > 0):
                a, b = q[i][wl], q[i + 1][wr]
                if a is not None and b is None:
                    q[i + 1][wr] = a + qphys[so] - qphys[si]
                    changed = True
                elif b is not None and a is None:
                    q[i][wl] = b - qphys[so] + qphys[si]
                    changed = True
                elif a is not None and a + qphys[so] != b + qphys[si]:
                    raise ValueError("MPO is not U(1) symmetric")
    return [np.array([0 if v is None else v for v in b]) for b in q]


def allowed3(Vl, Vr, qphys):
    """Mask of the allowed entries of A[a, s, b]: q(a) + qp(s) == q(b)."""
    qa, qb = Vl.basis_charges(), Vr.basis_charges()
    qs = np.asarray(qphys)
    return (qa[:, None, None] + qs[None, :, None]) == qb[None, None, :]


def allowed_env(V, qw):
    """Mask of the allowed entries of an environment E[a', w, a]: q(a') == q(a) + qw(w)."""
    q = V.basis_charges()
    return q[:, None, None] == (q[None, None, :] + np.asarray(qw)[None, :, None])


def _blocks2(Vl, Vr, qp1, qp2):
    d1, d2 = len(qp1), len(qp2)
    out = []
    for ib, qb in enumerate(Vr.charges):
        for s in range(d1 * d2):
            qs = qp1[s % d1] + qp2[s // d1]
            for ia, qa in enumerate(Vl.charges):
                if qa + qs == qb:
                    out.append((ia, s, ib))
    return out


def pack2(X, Vl, Vr, qp1, qp2):
    """Dense charge-sorted x[a, s1, s2, b] -> allowed blocks, ia fastest, then
    s = s1 + d1*s2, then ib; each block column-major."""
    d1 = len(qp1)
    parts = []
    for ia, s, ib in _blocks2(Vl, Vr, qp1, qp2):
        oa, da = Vl.offsets[ia], Vl.dims[ia]
        ob, db = Vr.offsets[ib], Vr.dims[ib]
        parts.append(X[oa:oa + da, s % d1, s // d1, ob:ob + db].ravel(order="F"))
    return np.concatenate(parts) if parts else np.zeros(0)


def unpack2(x, Vl, Vr, qp1, qp2):
    d1, d2 = len(qp1), len(qp2)
    X = np.zeros((Vl.dim, d1, d2, Vr.dim))
    o = 0
    for ia, s, ib in _blocks2(Vl, Vr, qp1, qp2):
        oa, da = Vl.offsets[ia], Vl.dims[ia]
        ob, db = Vr.offsets[ib], Vr.dims[ib]
        X[oa:oa + da, s % d1, s // d1, ob:ob + db] = x[o:o + da * db].reshape(da, db, order="F")
        o += da * db
    return X


def ac2_prime_blocks(X, W1, W2, L, R, Vl, Vr, qp1, qp2, qwl, qwr):
    """ac2_prime (derivatives.jl:20-22) block by block, the way a block-sparse
    tensor library contracts U1Space tensors: for every allowed output block
    (a', s1', s2', b') sum over MPO channels (w, w2) and input blocks with
    matrix products of the sector blocks only.  Same pairwise order as the
    dense restatement: (L x) first, then the MPO, then R."""
    d1, d2 = len(qp1), len(qp2)
    P = d1 * d2
    wl, wr = W1.shape[0], W2.shape[2]
    # O[w, w2, so, si] = sum_m W1[w, s1', m, s1] W2[m, s2', w2, s2], s = s1 + d1*s2
    O = np.einsum("wamb,mcxd->wxcadb", W1, W2).reshape(wl, wr, P, P)
    Y = np.zeros_like(X)
    nl, nr = len(Vl.charges), len(Vr.charges)

    def blk(V, i):
        return slice(V.offsets[i], V.offsets[i] + V.dims[i])

    qs = [qp1[s % d1] + qp2[s // d1] for s in range(P)]
    # T1[(ia', w, si, ib)] = L[a', w, a] x[a, si, b]
    T1 = {}
    for ib in range(nr):
        for si in range(P):
            ia = Vl.find(Vr.charges[ib] - qs[si])
            if ia < 0:
                continue
            xb = X[blk(Vl, ia), si % d1, si // d1, blk(Vr, ib)]
            for w in range(wl):
                iap = Vl.find(Vl.charges[ia] + int(qwl[w]))
                if iap < 0:
                    continue
                T1[(iap, w, si, ib)] = L[blk(Vl, iap), w, blk(Vl, ia)] @ xb
    for ibp in range(nr):
        for so in range(P):
            iap = Vl.find(Vr.charges[ibp] - qs[so])
            if iap < 0:
                continue
            acc = np.zeros((Vl.dims[iap], Vr.dims[ibp]))
            for w2 in range(wr):
                ib = Vr.find(Vr.charges[ibp] - int(qwr[w2]))
                if ib < 0:
                    continue
                T3 = np.zeros((Vl.dims[iap], Vr.dims[ib]))
                nz = False
                for w in range(wl):
                    for si in range(P):
                        c = O[w, w2, so, si]
                        if c == 0.0 or (iap, w, si, ib) not in T1:
                            continue
                        T3 += c * T1[(iap, w, si, ib)]
                        nz = True
                if nz:
                    acc += T3 @ R[blk(Vr, ibp), w2, blk(Vr, ib)].T
            Y[blk(Vl, iap), so % d1, so // d1, blk(Vr, ibp)] = acc
    return Y


def u1_split(X, Vl, Vr, qp1, qp2, trunc, side):
    """Per-sector SVD of x[(a s1), (s2 b)] with the cross-sector
    MPSTruncation rule and normalize!(s).  side 0: A = u, B = s v; side 1:
    A = u s, B = v.  Returns (A, S, B, Vm, err) with A [Dl, d1, Dm], B
    [Dm, d2, Dr] in the new charge-sorted basis (sectors in increasing charge,
    rows ordered (s1, a), columns (s2, b) inside a sector)."""
    d1, d2 = len(qp1), len(qp2)
    Dl, Dr = Vl.dim, Vr.dim
    cands = sorted({qa + qp1[s1] for qa in Vl.charges for s1 in range(d1)})
    secs = []
    for qc in cands:
        rows = [(s1, ia) for s1 in range(d1) for ia in range(len(Vl.charges))
                if Vl.charges[ia] + qp1[s1] == qc]
        cols = [(s2, ib) for s2 in range(d2) for ib in range(len(Vr.charges))
                if Vr.charges[ib] - qp2[s2] == qc]
        if not rows or not cols:
            continue
        r = sum(Vl.dims[ia] for _, ia in rows)
        c = sum(Vr.dims[ib] for _, ib in cols)
        M = np.zeros((r, c))
        ro = 0
        for s1, ia in rows:
            co = 0
            for s2, ib in cols:
                M[ro:ro + Vl.dims[ia], co:co + Vr.dims[ib]] = X[
                    Vl.offsets[ia]:Vl.offsets[ia] + Vl.dims[ia], s1, s2,
                    Vr.offsets[ib]:Vr.offsets[ib] + Vr.dims[ib]]
                co += Vr.dims[ib]
            ro += Vl.dims[ia]
        u, s, vh = np.linalg.svd(M, full_matrices=False)
        secs.append(dict(q=qc, rows=rows, cols=cols, u=u, s=s, vh=vh, keep=0))
    allv = np.concatenate([S["s"] for S in secs])
    nrm = np.linalg.norm(allv)
    cand = [(S["s"][i], k, i) for k, S in enumerate(secs) for i in range(len(S["s"]))
            if S["s"][i] >= trunc.eps * nrm]
    cand.sort(key=lambda t: (-t[0], t[1], t[2]))
    cand = cand[:trunc.D]
    for v, k, i in cand:
        secs[k]["keep"] = max(secs[k]["keep"], i + 1)
    kept2 = sum(float(np.sum(S["s"][:S["keep"]] ** 2)) for S in secs)
    err = float(np.sqrt(sum(float(np.sum(S["s"][S["keep"]:] ** 2)) for S in secs)))
    knorm = np.sqrt(kept2)
    Vm = Leg([(S["q"], S["keep"]) for S in secs if S["keep"] > 0])
    Dm = Vm.dim
    A = np.zeros((Dl, d1, Dm))
    B = np.zeros((Dm, d2, Dr))
    Sout = []
    for S in secs:
        k = S["keep"]
        if k == 0:
            continue
        im = Vm.find(S["q"])
        om = Vm.offsets[im]
        sv = S["s"][:k] / knorm
        Sout.append(sv)
        U = S["u"][:, :k]
        V = S["vh"][:k, :]
        if side == 0:
            V = sv[:, None] * V
        else:
            U = U * sv[None, :]
        ro = 0
        for s1, ia in S["rows"]:
            A[Vl.offsets[ia]:Vl.offsets[ia] + Vl.dims[ia], s1, om:om + k] = U[ro:ro + Vl.dims[ia]]
            ro += Vl.dims[ia]
        co = 0
        for s2, ib in S["cols"]:
            B[om:om + k, s2, Vr.offsets[ib]:Vr.offsets[ib] + Vr.dims[ib]] = V[:, co:co + Vr.dims[ib]]
            co += Vr.dims[ib]
    return A, np.concatenate(Sout), B, Vm, err


def random_u1_state(L, N, D, qphys, rng):
    """Bond legs and iid N(0,1) allowed blocks: bond i holds the charges that
    i sites can carry with N in total; dimensions share D in proportion to
    the number of product states, capped by min(left states, right states)."""
    legs = []
    for i in range(L + 1):
        left, right = sector_counts(i, qphys), sector_counts(L - i, qphys)
        caps = {q: min(c, right[N - q]) for q, c in left.items() if right.get(N - q, 0) > 0}
        tot = sum(caps.values())
        dims = caps if tot <= D else {q: max(1, min(c, int(D * c / tot))) for q, c in caps.items()}
        legs.append(Leg(dims))
    mps = []
    for i in range(L):
        A = np.zeros((legs[i].dim, len(qphys), legs[i + 1].dim))
        for ia, qa in enumerate(legs[i].charges):
            for s, qs in enumerate(qphys):
                ib = legs[i + 1].find(qa + qs)
                if ib < 0:
                    continue
                oa, da = legs[i].offsets[ia], legs[i].dims[ia]
                ob, db = legs[i + 1].offsets[ib], legs[i + 1].dims[ib]
                A[oa:oa + da, s, ob:ob + db] = rng.standard_normal((da, db))
        mps.append(A)
    return mps, legs


class U1OracleEnv(OracleEnv):
    """OracleEnv on charge-sorted dense tensors plus the bond legs."""

    def __init__(self, mpo, mps, legs, qphys, schur=True):
        self.legs = list(legs)
        self.qphys = list(qphys)
        super().__init__(mpo, mps, schur=schur)

    def right_canonicalize(self):
        """Exact two-site splits (side 1) from the right, normalising."""
        L = len(self.mps)
        for site in range(L - 1, 0, -1):
            x2 = np.tensordot(self.mps[site - 1], self.mps[site], axes=([2], [0]))

            class T:
                D = self.legs[site].dim
                eps = 1e-14
            A, S, B, Vm, _ = u1_split(x2, self.legs[site - 1], self.legs[site + 1], self.qphys,
                                      self.qphys, T, 1)
            self.mps[site - 1], self.mps[site], self.legs[site] = A, B, Vm
        self.init_hstorage(center=1)


def _u1_bond(env, site, trunc, eig_maxiter, eig_tol, direction):
    mps, mpo, hs = env.mps, env.mpo, env.hstorage
    A, B = mps[site - 1], mps[site]
    x2 = np.tensordot(A, B, axes=([2], [0]))
    shape = x2.shape
    W1, W2, L, R = mpo[site - 1], mpo[site], hs[site - 1], hs[site + 1]

    def f(v):
        return ac2_prime(v.reshape(shape, order="F"), W1, W2, L, R).ravel(order="F")

    E, vec, info, k = simple_lanczos_solver(f, x2.ravel(order="F"), eig_maxiter, eig_tol)
    vec = vec.reshape(shape, order="F")
    Au, S, Bv, Vm, err = u1_split(vec, env.legs[site - 1], env.legs[site + 1], env.qphys,
                                  env.qphys, trunc, 0 if direction == "left" else 1)
    usv = np.tensordot(Au, Bv, axes=([2], [0]))
    delta = abs(1 - abs(np.vdot(usv, x2)))
    mps[site - 1], mps[site] = Au, Bv
    env.legs[site] = Vm
    if direction == "left":
        env.updateleft_(site)
    else:
        env.updateright_(site + 1)
    return E, delta, k


def u1_dmrg2_sweep(env, trunc, eig_maxiter=10, eig_tol=1e-12):
    """sweep!(m, ::DMRG2) (dmrgexcited.jl:219-223, dmrg.jl:89-144) on U(1) tensors."""
    Es, delta = [], 0.0
    L = len(env.mps)
    for site in range(1, L - 1):
        E, dl, _ = _u1_bond(env, site, trunc, eig_maxiter, eig_tol, "left")
        Es.append(E)
        delta = max(delta, dl)
    for site in range(L - 1, 0, -1):
        E, dl, _ = _u1_bond(env, site, trunc, eig_maxiter, eig_tol, "right")
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta

