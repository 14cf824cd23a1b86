"""U(1)-symmetric (charge-conserving) two-site DMRG on the device.

The reference runs its DMRG code unchanged on TensorKit tensors with
``U1Space`` legs (``heisenberg_xxz_chain``, utilities/models.jl:47, with the
physical charges of ``abelian_matrix_from_dense``,
auxiliary/abelianmatrix.jl:112-124: basis state i has charge i).  TensorKit
then contracts and factorises sector by sector.  Here:

- a leg is a ``U1Space`` (charge-sorted sector table);
- MPS tensors A[a, s, b] and environments L[a', w, a] are dense device
  tensors in the charge-sorted bases, exactly zero outside the allowed blocks
  (q(a) + qp(s) == q(b); q(a') == q(a) + qw(w));
- the two-site vector is packed (allowed blocks only);
- ``ac2_prime``, the environment updates, the two-site product and the
  per-sector truncated SVD run in libfmpt's grouped block-sparse engine:
  one persistent launch per contraction over all (sector, w, w') blocks.

Everything is FP64, the reference's Float64 path.
"""

import ctypes

import numpy as np

from ._native import F64, U1SpaceC, lib
from .auxiliary import MPSTruncation, dot
from .device import DeviceTensor, default_handle, to_host_mpo
from .envs import _mpo_tensors, l_LL, r_RR
from .mps import OneBased

__all__ = ["U1Space", "U1FiniteMPS", "U1ExpectationCache", "U1HeffOp", "u1_randommps",
           "u1_environments", "mpo_channel_charges", "u1_twosite", "u1_split", "u1_pack2",
           "u1_unpack2", "u1_updateleft", "u1_updateright", "u1_leftsweep_", "u1_rightsweep_",
           "u1_expectation", "sector_counts"]


def _cints(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int * max(len(vals), 1))(*vals)


class U1Space:
    """U1Space(q1 => d1, q2 => d2, ...): sectors sorted by charge, zero-
    dimensional sectors dropped.  ``offsets`` locate each sector in the
    charge-sorted basis."""

    def __init__(self, sectors):
        items = sectors.items() if isinstance(sectors, dict) else sectors
        merged = {}
        for q, d in items:
            q, d = int(q), int(d)
            if d < 0:
                raise ValueError("negative sector dimension")
            if q in merged:
                raise ValueError("duplicate charge %d" % q)
            if d:
                merged[q] = d
        if not merged:
            raise ValueError("empty U1Space")
        self.charges = tuple(sorted(merged))
        self.dims = tuple(merged[q] for q in self.charges)
        offs, o = [], 0
        for d in self.dims:
            offs.append(o)
            o += d
        self.offsets = tuple(offs)
        self.dim = o
        self._q = _cints(self.charges)
        self._d = _cints(self.dims)
        self.c = U1SpaceC(len(self.charges), ctypes.cast(self._q, ctypes.POINTER(ctypes.c_int)),
                          ctypes.cast(self._d, ctypes.POINTER(ctypes.c_int)))

    @property
    def ref(self):
        return ctypes.byref(self.c)

    def sector(self, q):
        """(offset, dim) of charge q, or None."""
        try:
            i = self.charges.index(int(q))
        except ValueError:
            return None
        return self.offsets[i], self.dims[i]

    def basis_charges(self):
        return np.repeat(np.asarray(self.charges), self.dims)

    def __eq__(self, other):
        return isinstance(other, U1Space) and self.charges == other.charges and \
            self.dims == other.dims

    def __hash__(self):
        return hash((self.charges, self.dims))

    def __repr__(self):
        return "U1Space(%s)" % ", ".join("%d=>%d" % (q, d) for q, d in zip(self.charges, self.dims))


def sector_counts(n_sites, qphys):
    """Number of product basis states of n_sites sites per total charge."""
    c = {0: 1}
    for _ in range(n_sites):
        nxt = {}
        for q, k in c.items():
            for qp in qphys:
                nxt[q + qp] = nxt.get(q + qp, 0) + k
        c = nxt
    return c


def mpo_channel_charges(Ws, qphys):
    """Charges of every MPO bond channel: qw(wr) = qw(wl) + qp(s') - qp(s) for
    each nonzero W[wl, s', wr, s], propagated from the left boundary channel
    (charge 0) in both directions until nothing changes.  Returns L+1 integer
    arrays (bond i = left of site i, 1-based as OneBased)."""
    L = len(Ws)
    qp = [int(q) for q in qphys]
    q = [[None] * Ws[0].shape[0]] + [[None] * W.shape[2] for W in Ws]
    q[0][0] = 0
    nz = [np.argwhere(np.abs(np.asarray(W)) > 0) for W in Ws]
    changed = True
    while changed:
        changed = False
        for i in range(L):
            for wl, so, wr, si in nz[i]:
                a, b = q[i][wl], q[i + 1][wr]
                if a is not None and b is None:
                    q[i + 1][wr] = a + qp[so] - qp[si]
                    changed = True
                elif b is not None and a is None:
                    q[i][wl] = b - qp[so] + qp[si]
                    changed = True
                elif a is not None and a + qp[so] != b + qp[si]:
                    raise ValueError("MPO tensor %d does not conserve the U(1) charge" % (i + 1))
    return OneBased([np.array([0 if v is None else v for v in b], dtype=np.int64) for b in q])


class U1FiniteMPS:
    """FiniteMPS (mps/finitemps.jl:19-22) with U1Space virtual legs:
    ``spaces[i]`` is the bond left of site i (i = 1..L+1), ``qphys`` the
    physical charges."""

    def __init__(self, data, spaces, qphys=(0, 1), svectors=None):
        self.data = OneBased(data)
        self.spaces = OneBased(spaces)
        self.qphys = tuple(int(q) for q in qphys)
        self._qp = _cints(self.qphys)
        L = len(self.data)
        if len(self.spaces) != L + 1:
            raise ValueError("need L+1 bond spaces")
        self.s = OneBased(svectors if svectors is not None else [None] * (L + 1))
        for i in range(1, L + 1):
            self._check(i, self.data[i])

    def _check(self, i, A):
        want = (self.spaces[i].dim, len(self.qphys), self.spaces[i + 1].dim)
        if tuple(A.shape) != want:
            raise ValueError("SpaceMismatch: site %d tensor %s vs spaces %s" % (i, A.shape, want))

    def __len__(self):
        return len(self.data)

    def __getitem__(self, i):
        return self.data[i]

    def set_site(self, i, A, left=None, right=None):
        """mps[i] = A, optionally with new bond spaces on either side."""
        if left is not None:
            self.spaces[i] = left
        if right is not None:
            self.spaces[i + 1] = right
        self._check(i, A)
        self.data[i] = A

    @property
    def dtype(self):
        return np.dtype(np.float64)

    @property
    def handle(self):
        return self.data[1].h

    @property
    def total_charge(self):
        return self.spaces[len(self) + 1].charges[0]

    def bond_dimensions(self):
        return [self.spaces[i].dim for i in range(1, len(self) + 2)]

    def to_numpy(self):
        return [A.numpy() for A in self.data]


def _random_blocks(Vl, Vr, qphys, rng):
    A = np.zeros((Vl.dim, len(qphys), Vr.dim))
    for ql, ol, dl in zip(Vl.charges, Vl.offsets, Vl.dims):
        for s, qs in enumerate(qphys):
            sec = Vr.sector(ql + qs)
            if sec is None:
                continue
            orr, dr = sec
            A[ol:ol + dl, s, orr:orr + dr] = rng.standard_normal((dl, dr))
    return A


def random_u1_tensors(L, N, D, qphys=(0, 1), rng=None):
    """Host side of u1_randommps: bond spaces and iid N(0,1) allowed blocks
    (mps/initializers.jl:4-26 with U1Space legs).  Bond i holds the charges
    reachable by i sites with N in total; sector dimensions share D in
    proportion to the number of product states, each capped by the exact
    Hilbert-space dimension min(left states, right states)."""
    rng = np.random.default_rng(rng)
    qphys = tuple(int(q) for q in qphys)
    spaces = []
    for i in range(L + 1):
        left = sector_counts(i, qphys)
        right = sector_counts(L - i, qphys)
        caps = {q: min(c, right[N - q]) for q, c in left.items() if right.get(N - q, 0) > 0}
        if not caps:
            raise ValueError("no state with total charge %d" % N)
        tot = sum(caps.values())
        if tot <= D:
            dims = caps
        else:
            dims = {q: max(1, min(c, int(D * c / tot))) for q, c in caps.items()}
        spaces.append(U1Space(dims))
    tensors = [_random_blocks(spaces[i], spaces[i + 1], qphys, rng) for i in range(L)]
    return tensors, spaces


def u1_randommps(L, N, D, qphys=(0, 1), rng=None, handle=None, canonical=True, method="dm"):
    """randommps with U1Space legs and total charge N, right-canonicalised and
    normalised (canonicalize!(normalize=true), mps/orth.jl:40-49) by exact
    two-site splits from the right."""
    handle = handle or default_handle()
    tensors, spaces = random_u1_tensors(L, N, D, qphys, rng)
    psi = U1FiniteMPS([DeviceTensor.from_numpy(A, handle) for A in tensors], spaces, qphys)
    if canonical:
        u1_right_canonicalize_(psi, method)
    return psi


def u1_right_canonicalize_(psi, method="dm"):
    """Right-canonical form through two-site splits (side 1) that keep every
    nonzero singular value, sweeping from the right; the last split
    normalises the state.  ``method`` as in u1_split."""
    L = len(psi)
    for i in range(L - 1, 0, -1):
        Vl, Vm, Vr = psi.spaces[i], psi.spaces[i + 1], psi.spaces[i + 2]
        x = u1_twosite(psi[i], psi[i + 1], Vl, Vm, Vr, psi.qphys, psi.qphys)
        trunc = MPSTruncation(Vm.dim, 1e-14)
        A, S, B, Vnew, _ = u1_split(x, Vl, Vr, psi.qphys, psi.qphys, trunc, 1, method)
        psi.set_site(i + 1, B, left=Vnew)
        psi.set_site(i, A)
        psi.s[i + 1] = S
    return psi


# ------------------------------------------------------------ primitives
def _phys(qphys):
    return len(qphys), _cints(qphys)


def u1_twosite_size(Vl, Vr, qp1, qp2):
    n = ctypes.c_int64()
    d1, q1 = _phys(qp1)
    d2, q2 = _phys(qp2)
    st = lib().fmpt_u1_twosite_size(None, Vl.ref, Vr.ref, d1, q1, d2, q2, ctypes.byref(n))
    if st != 0:
        raise ValueError("u1_twosite_size: status %d" % st)
    return n.value


def u1_twosite(A, B, Vl, Vm, Vr, qp1, qp2):
    """Packed x[a, s1, s2, b] = sum_m A[a, s1, m] B[m, s2, b] (dmrg.jl:98)."""
    h = A.h
    n = u1_twosite_size(Vl, Vr, qp1, qp2)
    x = DeviceTensor((n,), np.float64, h)
    d1, q1 = _phys(qp1)
    d2, q2 = _phys(qp2)
    h.check(lib().fmpt_u1_twosite(h.ptr, F64, A.ptr, B.ptr, x.ptr, Vl.ref, Vm.ref, Vr.ref, d1, q1,
                                  d2, q2))
    return x


def u1_pack2(X, Vl, Vr, qp1, qp2):
    """Dense charge-sorted x[a, s1, s2, b] (device) -> packed blocks."""
    h = X.h
    n = u1_twosite_size(Vl, Vr, qp1, qp2)
    y = DeviceTensor((n,), np.float64, h)
    d1, q1 = _phys(qp1)
    d2, q2 = _phys(qp2)
    h.check(lib().fmpt_u1_pack2(h.ptr, F64, X.ptr, y.ptr, Vl.ref, Vr.ref, d1, q1, d2, q2, 0))
    return y


def u1_unpack2(x, Vl, Vr, qp1, qp2):
    """Packed -> dense charge-sorted x[a, s1, s2, b] (zeros elsewhere)."""
    h = x.h
    d1, q1 = _phys(qp1)
    d2, q2 = _phys(qp2)
    X = DeviceTensor((Vl.dim, d1, d2, Vr.dim), np.float64, h)
    h.check(lib().fmpt_u1_pack2(h.ptr, F64, x.ptr, X.ptr, Vl.ref, Vr.ref, d1, q1, d2, q2, 1))
    return X


def u1_split(x, Vl, Vr, qp1, qp2, trunc, side, method="gesvd"):
    """Truncated, normalised two-site split (stable_tsvd! + normalize!(s) of
    DMRG2 with TensorKit's cross-sector truncation).  ``method`` "gesvd": an
    SVD per sector; "dm": the density-matrix form (batched eigensolves, see
    include/fmpt.h).  Returns (A [Dl, d1, Dm], S [Dm], B [Dm, d2, Dr], Vm, err)."""
    if method not in ("gesvd", "dm"):
        raise ValueError("method must be 'gesvd' or 'dm'")
    h = x.h
    d1, q1 = _phys(qp1)
    d2, q2 = _phys(qp2)
    cap_d = max(1, min(trunc.D, Vl.dim * d1, d2 * Vr.dim))
    A = DeviceTensor((Vl.dim, d1, cap_d), np.float64, h)
    S = DeviceTensor((cap_d,), np.float64, h)
    B = DeviceTensor((cap_d, d2, Vr.dim), np.float64, h)
    cap = len(Vl.charges) * d1 + 1
    ns = ctypes.c_int()
    qo = (ctypes.c_int * cap)()
    do = (ctypes.c_int * cap)()
    err = ctypes.c_double()
    h.check(lib().fmpt_u1_split(h.ptr, F64, x.ptr, Vl.ref, Vr.ref, d1, q1, d2, q2, int(trunc.D),
                                float(trunc.eps), int(side), 0 if method == "gesvd" else 1,
                                A.ptr, S.ptr, B.ptr, cap,
                                ctypes.byref(ns), qo, do, ctypes.byref(err)))
    Vm = U1Space([(qo[i], do[i]) for i in range(ns.value)])
    A.view_as((Vl.dim, d1, Vm.dim))
    S.view_as((Vm.dim,))
    B.view_as((Vm.dim, d2, Vr.dim))
    return A, S, B, Vm, err.value


def _u1_env(right, hold, A, W, B, Vl, Vr, qp, qwl, qwr):
    h = A.h
    W = np.asarray(W, dtype=np.float64)
    wl, d, wr = W.shape[0], W.shape[1], W.shape[2]
    buf = to_host_mpo(W, np.float64)
    dd, qpc = _phys(qp)
    if dd != d:
        raise ValueError("DimensionMismatch: physical charges vs MPO")
    out_shape = (Vl.dim, wl, Vl.dim) if right else (Vr.dim, wr, Vr.dim)
    hnew = DeviceTensor(out_shape, np.float64, h)
    fn = lib().fmpt_u1_updateright if right else lib().fmpt_u1_updateleft
    h.check(fn(h.ptr, F64, hold.ptr, A.ptr, buf.ctypes.data, B.ptr, hnew.ptr, Vl.ref, Vr.ref, d,
               qpc, wl, _cints(qwl), wr, _cints(qwr)))
    return hnew


def u1_updateleft(hold, A, W, B, Vl, Vr, qp, qwl, qwr):
    """updateleft(hold, A, W, B) (mpo/transfer.jl:31-34) on U(1) tensors."""
    return _u1_env(False, hold, A, W, B, Vl, Vr, qp, qwl, qwr)


def u1_updateright(hold, A, W, B, Vl, Vr, qp, qwl, qwr):
    """updateright(hold, A, W, B) (mpo/transfer.jl:26-29) on U(1) tensors."""
    return _u1_env(True, hold, A, W, B, Vl, Vr, qp, qwl, qwr)


class U1HeffOp:
    """Block-sparse two-site ac2_prime operator on packed vectors (fmpt_op)."""

    def __init__(self, hleft, hright, W1, W2, Vl, Vr, qp1, qp2, qwl, qwm, qwr):
        self.h = hleft.h
        self.hleft, self.hright = hleft, hright
        W1 = np.asarray(W1, dtype=np.float64)
        W2 = np.asarray(W2, dtype=np.float64)
        self._bufs = [to_host_mpo(W1, np.float64), to_host_mpo(W2, np.float64)]
        d1, q1 = _phys(qp1)
        d2, q2 = _phys(qp2)
        op = ctypes.c_void_p()
        self.ptr = None
        self.h.check(lib().fmpt_u1_op_ac2(
            self.h.ptr, F64, self._bufs[0].ctypes.data, self._bufs[1].ctypes.data, hleft.ptr,
            hright.ptr, Vl.ref, Vr.ref, d1, q1, d2, q2, W1.shape[0], _cints(qwl), W1.shape[2],
            _cints(qwm), W2.shape[2], _cints(qwr), ctypes.byref(op)))
        self.ptr = op
        self.n = int(lib().fmpt_op_size(op))
        self.shape = (self.n,)

    def tile(self):
        """Output tile edge the grouped kernel runs this operator with (autotuned)."""
        return int(lib().fmpt_op_tile(self.ptr))

    def flops(self):
        f = ctypes.c_double()
        self.h.check(lib().fmpt_op_flops(self.ptr, ctypes.byref(f)))
        return f.value

    def __del__(self):
        try:
            if self.ptr:
                lib().fmpt_op_destroy(self.ptr)
        except Exception:
            pass
        self.ptr = None

    def __call__(self, x, out=None):
        if tuple(x.shape) != self.shape:
            raise ValueError("DimensionMismatch: x %s vs operator %s" % (x.shape, self.shape))
        y = out if out is not None else DeviceTensor(self.shape, np.float64, self.h)
        self.h.check(lib().fmpt_op_apply(self.ptr, x.ptr, y.ptr))
        return y

    def set_projectors(self, projectors):
        """Compose with _project! (dmrgexcited.jl:1-6) on packed vectors: after
        every application y -= dot(y, p) p for each packed device vector p."""
        for p in projectors:
            if tuple(p.shape) != self.shape or p.dtype != np.float64:
                raise ValueError("DimensionMismatch: projector %s vs %s" % (p.shape, self.shape))
        self._proj = list(projectors)
        arr = (ctypes.c_void_p * max(1, len(self._proj)))(*[p.ptr for p in self._proj])
        self.h.check(lib().fmpt_op_set_projectors(self.ptr, len(self._proj), arr))

    def lanczos(self, x0, kmax=10, btol=1e-8, reorth=False):
        """simple_lanczos_solver(f, x0, "SR", kmax, btol) on packed vectors."""
        out = DeviceTensor(self.shape, np.float64, self.h)
        ev, info, it = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        self.h.check(lib().fmpt_lanczos_ground(self.ptr, x0.ptr, int(kmax), float(btol),
                                               1 if reorth else 0, ctypes.byref(ev), out.ptr,
                                               ctypes.byref(info), ctypes.byref(it)))
        return ev.value, out, info.value, it.value


# ----------------------------------------------------------- environments
class U1ExpectationCache:
    """ExpectationCache (envs/finiteenv.jl:51-69) for a U1FiniteMPS: dense
    charge-sorted environments, MPO channel charges per bond."""

    def __init__(self, mpo, mps):
        L = len(mps)
        Ws, schur = _mpo_tensors(mpo, L)
        if any(np.iscomplexobj(W) for W in Ws):
            raise TypeError("U(1) path: real MPO tensors only")
        self.h_input = mpo
        self.dtype = np.dtype(np.float64)
        self.mpo = OneBased([np.asarray(W, dtype=np.float64) for W in Ws])
        self.qw = mpo_channel_charges(self.mpo.tolist(), mps.qphys)
        self.mps = mps
        self.schur = schur
        self.precision = "fp64"
        self.hstorage = OneBased([None] * (L + 1))
        u1_init_hstorage_(self, 1)

    @property
    def state(self):
        return self.mps

    @property
    def h(self):
        return self.mpo

    @property
    def env(self):
        return self.hstorage


def u1_init_hstorage_(m, center=1):
    """init_hstorage! (finiteenv.jl:1-21)."""
    L = len(m.mps)
    hd = m.mps.handle
    hs = m.hstorage
    if m.mps.spaces[1].charges != (0,) or m.mps.spaces[1].dims != (1,):
        raise ValueError("left boundary leg must be U1Space(0 => 1)")
    if len(m.mps.spaces[L + 1].charges) != 1 or m.mps.spaces[L + 1].dims != (1,):
        raise ValueError("right boundary leg must hold one charge of dimension 1")
    hs[L + 1] = r_RR(m.mpo[L].shape[2], m.dtype, hd, m.schur)
    hs[1] = l_LL(m.mpo[1].shape[0], m.dtype, hd, m.schur)
    for i in range(L, center, -1):
        u1_updateright_(m, i)
    for i in range(1, center):
        u1_updateleft_(m, i)
    return hs


def u1_environments(mpo, mps):
    return U1ExpectationCache(mpo, mps)


def u1_updateleft_(m, site):
    """updateleft!(env, site) (finiteenv.jl:72-74)."""
    psi = m.mps
    m.hstorage[site + 1] = u1_updateleft(m.hstorage[site], psi[site], m.mpo[site], psi[site],
                                         psi.spaces[site], psi.spaces[site + 1], psi.qphys,
                                         m.qw[site], m.qw[site + 1])


def u1_updateright_(m, site):
    """updateright!(env, site) (finiteenv.jl:76-78)."""
    psi = m.mps
    m.hstorage[site] = u1_updateright(m.hstorage[site + 1], psi[site], m.mpo[site], psi[site],
                                      psi.spaces[site], psi.spaces[site + 1], psi.qphys,
                                      m.qw[site], m.qw[site + 1])


# ----------------------------------------------------------------- DMRG2
def _u1_bond(m, site, alg, side):
    psi, hs = m.mps, m.hstorage
    qp = psi.qphys
    Vl, Vm, Vr = psi.spaces[site], psi.spaces[site + 1], psi.spaces[site + 2]
    x2 = u1_twosite(psi[site], psi[site + 1], Vl, Vm, Vr, qp, qp)
    op = U1HeffOp(hs[site], hs[site + 2], m.mpo[site], m.mpo[site + 1], Vl, Vr, qp, qp,
                  m.qw[site], m.qw[site + 1], m.qw[site + 2])
    E, vecs, info, k = op.lanczos(x2, alg.eig_maxiter, alg.eig_tol, alg.reorth)
    del op
    A, S, B, Vnew, err = u1_split(vecs, Vl, Vr, qp, qp, alg.trunc, side, alg.svd)
    usv = u1_twosite(A, B, Vl, Vnew, Vr, qp, qp)
    delta = abs(1 - abs(dot(usv, x2)))      # dmrg.jl:109-110
    del usv
    psi.set_site(site, A, right=Vnew)
    psi.set_site(site + 1, B, left=Vnew)
    if side == 0:
        u1_updateleft_(m, site)
    else:
        psi.s[site + 1] = S
        u1_updateright_(m, site + 1)
    if alg.verbosity > 2:
        print("bond %d (%s): E=%.15g lanczos k=%d D=%d" % (site, "left" if side == 0 else "right",
                                                           E, k, Vnew.dim))
    return E, delta


def _check_alg(alg):
    if getattr(alg, "precision", "fp64") != "fp64":
        raise ValueError("the U(1) path runs its contractions in FP64")
    if getattr(alg, "svd", "gesvd") not in ("gesvd", "dm"):
        raise ValueError("U(1) split: svd must be 'gesvd' or 'dm'")


def u1_leftsweep_(m, alg):
    """leftsweep!(m, ::DMRG2) (dmrg.jl:89-115) on U(1) tensors."""
    _check_alg(alg)
    Es, delta = [], 0.0
    for site in range(1, len(m.mps) - 1):
        E, dl = _u1_bond(m, site, alg, 0)
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def u1_rightsweep_(m, alg):
    """rightsweep!(m, ::DMRG2) (dmrg.jl:117-144) on U(1) tensors."""
    _check_alg(alg)
    Es, delta = [], 0.0
    for site in range(len(m.mps) - 1, 0, -1):
        E, dl = _u1_bond(m, site, alg, 1)
        Es.append(E)
        delta = max(delta, dl)
    return Es, delta


def u1_expectation(psi, h):
    """<psi|H|psi> for a U1FiniteMPS (mpohamiltonian/arithmetics.jl:5-19): a
    chain of left environment updates from l_LL, closed with r_RR."""
    L = len(psi)
    Ws, schur = _mpo_tensors(h, L)
    mpo = OneBased([np.asarray(W, dtype=np.float64) for W in Ws])
    qw = mpo_channel_charges(mpo.tolist(), psi.qphys)
    env = l_LL(mpo[1].shape[0], np.float64, psi.handle, schur)
    for i in range(1, L + 1):
        env = u1_updateleft(env, psi[i], mpo[i], psi[i], psi.spaces[i], psi.spaces[i + 1],
                            psi.qphys, qw[i], qw[i + 1])
    return float(env.numpy()[0, -1, 0])
