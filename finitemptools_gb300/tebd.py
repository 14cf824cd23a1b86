"""TEBD on the device: quantum gates applied to a right-canonical MPS with
singular vectors (circuit/apply_gates.jl, circuit/gate.jl, circuit/circuit.jl)
and the Trotter-Suzuki circuit of a nearest-neighbour Hamiltonian
(algorithms/tebd.jl:99-193).

A bond update keeps the reference's steps, all on the device: the gate
contracted into the n-site tensor (fmpt_apply_gate), the left singular
vectors multiplied in, the truncated split (cuSOLVER gesvd by default, the
density-matrix split with svd="dm"), and the new left tensor as theta * v^H,
which never divides by a singular value.

Gate operators are numpy arrays with 2N legs (out_1..out_N, in_1..in_N) or
square matrices over the fused physical index (first site fastest, the
column-major order of the MPS tensors).
"""

import numpy as np

from ._native import lib
from .auxiliary import default_truncation, dm_split, gemm, scale_rows, stable_tsvd
from .device import DeviceTensor, to_host_buffer
from .mps import canonicalize_

__all__ = ["QuantumGate", "QuantumCircuit", "apply_", "bond_evolution", "bond_evolution3",
           "bond_evolution4", "swap_gate", "move_", "trotter_propagator", "fuse_gates",
           "compute_step_size", "TEBDStepper", "HomogeneousTEBDCache",
           "InhomogeneousTEBDCache", "make_step_"]


class QuantumGate:
    """struct QuantumGate (gate.jl:8-20): positions are sorted on construction
    and the operator's legs permuted with them (_get_norm_order, :1-5)."""

    def __init__(self, positions, op, dims=None):
        pos = (int(positions),) if np.isscalar(positions) else tuple(int(p) for p in positions)
        N = len(pos)
        op = np.asarray(op)
        if op.ndim == 2:
            if dims is None:
                d = int(round(op.shape[0] ** (1.0 / N)))
                dims = (d,) * N
            if op.shape != (int(np.prod(dims)),) * 2:
                raise ValueError("gate matrix does not match the site dimensions")
            op = op.reshape(tuple(dims) * 2, order="F")
        if op.ndim != 2 * N:
            raise ValueError("a gate on %d sites needs %d legs" % (N, 2 * N))
        if list(pos) != sorted(pos):
            seq = list(np.argsort(pos, kind="stable"))
            pos = tuple(pos[i] for i in seq)
            op = op.transpose(seq + [s + N for s in seq])
        if len(set(pos)) != N:
            raise ValueError("repeated gate position")
        self.positions = pos
        self.op = op

    def matrix(self):
        """The gate as a P x P matrix over the fused index (first site fastest)."""
        N = len(self.positions)
        P = int(np.prod(self.op.shape[:N]))
        return self.op.reshape(P, P, order="F")

    def adjoint(self):
        """AdjointQuantumGate (gate.jl:39-52), materialised."""
        N = len(self.positions)
        return QuantumGate(self.positions, np.conj(self.op.transpose(list(range(N, 2 * N)) +
                                                                      list(range(N)))))

    def shift(self, i):
        return QuantumGate(tuple(p + i for p in self.positions), self.op)


class QuantumCircuit(list):
    """struct QuantumCircuit (circuit.jl:2-45): a list of gates applied in order."""

    def adjoint(self):
        return QuantumCircuit(g.adjoint() for g in reversed(self))

    def __mul__(self, other):
        """x * y applies y first (circuit.jl:45)."""
        return QuantumCircuit(list(other) + list(self))


# ---------------------------------------------------------------- gate fusion
# circuit/gate_fusion.jl: host algebra on the gates' small matrices (at most d^8 entries),
# done once per circuit before it is applied.
def _commute(a, b):
    """_is_commutative (gate_fusion.jl:3-25): gates on disjoint sites."""
    return not (set(a.positions) & set(b.positions))


def _embed(g, K, dims):
    """g's operator on the sorted sites K (a superset of g's), identity on the others."""
    N = len(K)
    if N > 8:
        raise ValueError("gate fusion supports at most 8 sites")
    out, inn = "abcdefgh"[:N], "ijklmnop"[:N]
    t = {k: i for i, k in enumerate(K)}
    subs = ["".join(out[t[p]] for p in g.positions) + "".join(inn[t[p]] for p in g.positions)]
    ops = [g.op]
    for i, k in enumerate(K):
        if k in g.positions:
            continue
        subs.append(out[i] + inn[i])
        ops.append(np.eye(dims[i], dtype=g.op.dtype))
    return np.einsum(",".join(subs) + "->" + out + inn, *ops)


def _try_mul(a, b):
    """try_mul_two_ops (gate_fusion.jl:357-362, with the per-arity contractions of
    :49-355): a applied after b as one gate, when the
    sites of one contain the other's; None otherwise.  The product sits on the larger
    site set."""
    big, small = (a, b) if len(a.positions) >= len(b.positions) else (b, a)
    if not set(small.positions) <= set(big.positions):
        return None
    K = big.positions
    dims = big.op.shape[:len(K)]
    for p, d in zip(small.positions, small.op.shape[:len(small.positions)]):
        if dims[K.index(p)] != d:
            raise ValueError("gates disagree on the dimension of site %d" % p)
    P = int(np.prod(dims))
    ma = _embed(a, K, dims).reshape(P, P, order="F")
    mb = _embed(b, K, dims).reshape(P, P, order="F")
    return QuantumGate(K, (ma @ mb).reshape(tuple(dims) * 2, order="F"))


def _absorb(gates, gate):
    """try_absorb_one_gate_by_mul! (gate_fusion.jl:364-374): multiply gate into the latest
    earlier gate it can join, passing only gates it commutes with."""
    for i in range(len(gates) - 1, -1, -1):
        r = _try_mul(gate, gates[i])
        if r is not None:
            gates[i] = r
            return True
        if not _commute(gates[i], gate):
            return False
    return False


def _fuse_pass(circuit):
    """try_absorb_by_mul_impl and _fuse_gate_impl (gate_fusion.jl:376-395): from the last gate to the second,
    each gate that an earlier one absorbs leaves the circuit."""
    b = list(circuit)
    for i in range(len(b) - 1, 0, -1):
        br = b[:i]
        if _absorb(br, b[i]):
            b = br + b[i + 1:]
    return QuantumCircuit(b)


def fuse_gates(circuit):
    """fuse_gates (gate_fusion.jl:397-400): one pass over the adjoint circuit (later gates
    absorbing earlier ones), then one over the circuit.  The result applies the same
    operator with fewer gates."""
    c = circuit if isinstance(circuit, QuantumCircuit) else QuantumCircuit(circuit)
    return _fuse_pass(_fuse_pass(c.adjoint()).adjoint())


# ---------------------------------------------------------------- bond updates
def _gate(G, x, Dl, P, Dr):
    """y[a, p', b] = sum_p G[p', p] x[a, p, b] on the device."""
    y = DeviceTensor(x.shape, x.dtype, x.h)
    buf = to_host_buffer(np.asarray(G), x.dtype)
    x.h.check(lib().fmpt_apply_gate(x.h.ptr, x.code, buf.ctypes.data, int(P), x.ptr, y.ptr,
                                    int(Dl), int(Dr)))
    return y


def _split(M, m, n, trunc, svd):
    """Truncated split keeping (s, v^H orthonormal rows, err)."""
    if svd == "dm":
        _, s, vt, err = dm_split(M, m, n, trunc, 1)
    else:
        _, s, vt, err = stable_tsvd(M, m, n, trunc)
    return s, vt, err


def _left_from(theta, m, n, vt):
    """u = theta * v^H: the new right-canonical left tensor (apply_gates.jl:16)."""
    k = vt.shape[0]
    return gemm(theta, vt, (m, k), m, k, n, tb="C")


def bond_evolution(G, s1, A1, s2, A2, trunc, svd="gesvd"):
    """bond_evolution (apply_gates.jl:11-18) -> (u, s, v, err); s2 is unused, as
    in the reference."""
    Dl, d1, Dm = A1.shape
    _, d2, Dr = A2.shape
    x2 = gemm(A1, A2, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, Dm)
    theta = _gate(G, x2, Dl, d1 * d2, Dr)
    th1 = scale_rows(theta.copy(), Dl, d1 * d2 * Dr, s1)
    s, vt, err = _split(th1, Dl * d1, d2 * Dr, trunc, svd)
    k = s.shape[0]
    u = _left_from(theta, Dl * d1, d2 * Dr, vt)
    return u.view_as((Dl, d1, k)), s, vt.view_as((k, d2, Dr)), err


def _next_split(v, s, dims, trunc, svd):
    """One more cut of v (rows scaled by s) -> (u2 = v v2^H, s2, v2, err)."""
    k1 = v.shape[0]
    d = dims[0]
    rest = int(np.prod(dims[1:]))
    n = v.size // k1
    v1 = scale_rows(v.copy(), k1, n, s)
    s2, v2, err = _split(v1, k1 * d, rest, trunc, svd)
    k2 = s2.shape[0]
    u2 = _left_from(v, k1 * d, rest, v2)
    return u2.view_as((k1, d, k2)), s2, v2, err


def bond_evolution3(G, s1, A1, s2, A2, s3, A3, trunc, svd="gesvd"):
    """bond_evolution3 (apply_gates.jl:21-33)."""
    Dl, d1, _ = A1.shape
    d2, d3, Dr = A2.shape[1], A3.shape[1], A3.shape[2]
    x = gemm(A1, A2, (Dl, d1, d2, A2.shape[2]), Dl * d1, d2 * A2.shape[2], A1.shape[2])
    x = gemm(x, A3, (Dl, d1, d2, d3, Dr), Dl * d1 * d2, d3 * Dr, A3.shape[0])
    P = d1 * d2 * d3
    theta = _gate(G, x, Dl, P, Dr)
    th1 = scale_rows(theta.copy(), Dl, P * Dr, s1)
    s, vt, e1 = _split(th1, Dl * d1, d2 * d3 * Dr, trunc, svd)
    k = s.shape[0]
    u = _left_from(theta, Dl * d1, d2 * d3 * Dr, vt).view_as((Dl, d1, k))
    u2, s2n, v2, e2 = _next_split(vt, s, (d2, d3, Dr), trunc, svd)
    return u, s, u2, s2n, v2.view_as((s2n.shape[0], d3, Dr)), max(e1, e2)


def bond_evolution4(G, s1, A1, s2, A2, s3, A3, s4, A4, trunc, svd="gesvd"):
    """bond_evolution4 (apply_gates.jl:35-52)."""
    Dl, d1, _ = A1.shape
    d2, d3, d4, Dr = A2.shape[1], A3.shape[1], A4.shape[1], A4.shape[2]
    x = gemm(A1, A2, (Dl, d1, d2, A2.shape[2]), Dl * d1, d2 * A2.shape[2], A1.shape[2])
    x = gemm(x, A3, (Dl, d1, d2, d3, A3.shape[2]), Dl * d1 * d2, d3 * A3.shape[2], A3.shape[0])
    x = gemm(x, A4, (Dl, d1, d2, d3, d4, Dr), Dl * d1 * d2 * d3, d4 * Dr, A4.shape[0])
    P = d1 * d2 * d3 * d4
    theta = _gate(G, x, Dl, P, Dr)
    th1 = scale_rows(theta.copy(), Dl, P * Dr, s1)
    s, vt, e1 = _split(th1, Dl * d1, d2 * d3 * d4 * Dr, trunc, svd)
    k = s.shape[0]
    u = _left_from(theta, Dl * d1, d2 * d3 * d4 * Dr, vt).view_as((Dl, d1, k))
    u2, s2n, v2, e2 = _next_split(vt, s, (d2, d3, d4, Dr), trunc, svd)
    u3, s3n, v3, e3 = _next_split(v2, s2n, (d3, d4, Dr), trunc, svd)
    return u, s, u2, s2n, u3, s3n, v3.view_as((s3n.shape[0], d4, Dr)), max(e1, e2, e3)


def _swap_matrix(d1, d2):
    """Permutation taking (s1 + d1 s2) to (s2 + d2 s1)."""
    G = np.zeros((d1 * d2, d1 * d2))
    for a in range(d1):
        for b in range(d2):
            G[b + d2 * a, a + d1 * b] = 1.0
    return G


def swap_gate(s1, A1, s2, A2, trunc, svd="gesvd"):
    """_swap_gate (apply_gates.jl:3-9): exchange two neighbouring sites."""
    Dl, d1, Dm = A1.shape
    _, d2, Dr = A2.shape
    x2 = gemm(A1, A2, (Dl, d1, d2, Dr), Dl * d1, d2 * Dr, Dm)
    theta = _gate(_swap_matrix(d1, d2), x2, Dl, d1 * d2, Dr)       # [Dl, d2, d1, Dr]
    th1 = scale_rows(theta.copy(), Dl, d1 * d2 * Dr, s1)
    s, vt, err = _split(th1, Dl * d2, d1 * Dr, trunc, svd)
    k = s.shape[0]
    u = _left_from(theta, Dl * d2, d1 * Dr, vt)
    return u.view_as((Dl, d2, k)), s, vt.view_as((k, d1, Dr)), err


def move_(psi, i, j, trunc, svd="gesvd"):
    """_move! (apply_gates.jl:54-73): carry site i to position j by swaps."""
    L = len(psi)
    if not (1 <= i <= L and 1 <= j <= L):
        raise IndexError("index out of range.")
    _ensure_svectors(psi)
    err = 0.0
    if i < j:
        for k in range(i, j):
            psi[k], psi.s[k + 1], psi[k + 1], e = swap_gate(psi.s[k], psi[k], psi.s[k + 1],
                                                            psi[k + 1], trunc, svd)
            err = max(err, e)
    elif i > j:
        for k in range(i, j, -1):
            psi[k - 1], psi.s[k], psi[k], e = swap_gate(psi.s[k - 1], psi[k - 1], psi.s[k],
                                                        psi[k], trunc, svd)
            err = max(err, e)
    return err


def _ensure_svectors(psi):
    """svectors_uninitialized(mps) && canonicalize!(mps) (apply_gates.jl:176)."""
    if any(psi.s[i] is None for i in range(1, len(psi) + 2)):
        canonicalize_(psi)


def _apply_impl(g, psi, trunc, svd):
    pos = g.positions
    G = g.matrix()
    if len(pos) == 1:                                   # apply_gates.jl:76-81
        key = pos[0]
        A = psi[key]
        Dl, d, Dr = A.shape
        psi[key] = _gate(G, A, Dl, d, Dr)
        return 0.0
    if len(pos) == 2:                                   # :83-98
        i, j = pos
        err = 0.0
        if i + 1 != j:
            err = max(err, move_(psi, i, j - 1, trunc, svd))
        psi[j - 1], psi.s[j], psi[j], e = bond_evolution(G, psi.s[j - 1], psi[j - 1], psi.s[j],
                                                         psi[j], trunc, svd)
        err = max(err, e)
        if i + 1 != j:
            err = max(err, move_(psi, j - 1, i, trunc, svd))
        return err
    if len(pos) == 3:                                   # :111-133
        i, j, k = pos
        nn = (j == i + 1 and k == j + 1)
        err = 0.0
        if not nn:
            err = max(err, move_(psi, i, j - 1, trunc, svd))
            err = max(err, move_(psi, k, j + 1, trunc, svd))
        (psi[j - 1], psi.s[j], psi[j], psi.s[j + 1], psi[j + 1], e) = bond_evolution3(
            G, psi.s[j - 1], psi[j - 1], psi.s[j], psi[j], psi.s[j + 1], psi[j + 1], trunc, svd)
        err = max(err, e)
        if not nn:
            err = max(err, move_(psi, j - 1, i, trunc, svd))
            err = max(err, move_(psi, j + 1, k, trunc, svd))
        return err
    if len(pos) == 4:                                   # :135-163
        i, j, k, l = pos
        nn = (j == i + 1 and k == j + 1 and l == k + 1)
        err = 0.0
        if not nn:
            err = max(err, move_(psi, i, j - 1, trunc, svd))
            err = max(err, move_(psi, k, j + 1, trunc, svd))
            err = max(err, move_(psi, l, j + 2, trunc, svd))
        (psi[j - 1], psi.s[j], psi[j], psi.s[j + 1], psi[j + 1], psi.s[j + 2], psi[j + 2],
         e) = bond_evolution4(G, psi.s[j - 1], psi[j - 1], psi.s[j], psi[j], psi.s[j + 1],
                              psi[j + 1], psi.s[j + 2], psi[j + 2], trunc, svd)
        err = max(err, e)
        if not nn:
            err = max(err, move_(psi, j - 1, i, trunc, svd))
            err = max(err, move_(psi, j + 2, l, trunc, svd))
            err = max(err, move_(psi, j + 1, k, trunc, svd))
        return err
    raise ValueError("only 4-body (or less) gates are currently allowed.")


def apply_(gates, psi, trunc=None, svd="gesvd"):
    """apply!(gate or circuit, mps; trunc) (apply_gates.jl:173-187): returns the
    truncation error of every gate."""
    trunc = trunc if trunc is not None else default_truncation()
    if isinstance(gates, QuantumGate):
        gates = [gates]
    _ensure_svectors(psi)
    errs = []
    for g in gates:
        if g.op.dtype.kind == "c" and psi.dtype != np.complex128:
            raise TypeError("a complex gate needs a complex MPS")
        errs.append(_apply_impl(g, psi, trunc, svd))
    return errs


# ------------------------------------------------------------ Trotter circuits
def _term_at(h, t):
    """A term's matrix at time t: h(t) for a time-dependent term, h itself otherwise."""
    return np.asarray(h(t) if callable(h) else h)


def _absorb_one_bodies(L, dims, bonds, sites):
    """_absorb_one_bodies (operators/quantumoperator.jl:221-258) on matrices:
    a one-body term of site i < L joins bond (i, i+1) as h (x) 1, the last
    site's joins (L-1, L) as 1 (x) h (first site fastest).  Terms may be
    functions of time; a sum with one of them is one too."""
    out = {k: (v if callable(v) else np.asarray(v)) for k, v in bonds.items()}
    for i, h in sites.items():
        if i < L:
            key, emb = (i, i + 1), (lambda m, e=np.eye(dims[i]): np.kron(e, m))
        else:
            key, emb = (i - 1, i), (lambda m, e=np.eye(dims[i - 2]): np.kron(m, e))
        if callable(h) or callable(out.get(key)):
            prev = out.get(key)
            out[key] = (lambda t, h=h, prev=prev, emb=emb:
                        emb(_term_at(h, t)) + (_term_at(prev, t) if prev is not None else 0.0))
        else:
            m = emb(np.asarray(h))
            out[key] = out[key] + m if key in out else m
    return out


def _expm_circuit(terms, t, dt):
    """_expm(ham, t, dt) (operators/quantumoperator.jl:198-219): one gate exp(dt h(t))
    per term."""
    import scipy.linalg
    return QuantumCircuit(QuantumGate(k, scipy.linalg.expm(dt * _term_at(h, t)))
                          for k, h in sorted(terms.items()))


def _propagator_2order(terms, tf, ti):
    """propagator_2order (tebd.jl:99-140): even/odd nearest-neighbour splitting
    (split_nn_ham, :24-38) or the symmetric generic form, the terms taken at the midpoint
    ti + dt/2."""
    dt = tf - ti
    tm = ti + dt / 2
    if all(len(k) == 2 and k[1] == k[0] + 1 for k in terms):
        even = {k: v for k, v in terms.items() if k[0] % 2 == 0}
        odd = {k: v for k, v in terms.items() if k[0] % 2 != 0}
        half = _expm_circuit(even, tm, dt / 2)
        return QuantumCircuit(list(half) + list(_expm_circuit(odd, tm, dt)) + list(half))
    tmp = _expm_circuit(terms, tm, dt / 2)
    return QuantumCircuit(list(tmp) + list(reversed(tmp)))


def _propagator_impl(terms, tf, ti, order):
    """_propagator_impl (tebd.jl:152-168): the Suzuki fractal recursion."""
    if order == 1:
        return _propagator_2order(terms, tf, ti)
    p = order - 1
    sp = 1.0 / (4.0 - 4.0 ** (1.0 / (2 * p + 1)))
    dt = tf - ti
    c = QuantumCircuit()
    c.extend(_propagator_impl(terms, ti + sp * dt, ti, p))
    c.extend(_propagator_impl(terms, ti + 2 * sp * dt, ti + sp * dt, p))
    c.extend(_propagator_impl(terms, ti + (1 - 2 * sp) * dt, ti + 2 * sp * dt, p))
    c.extend(_propagator_impl(terms, ti + (1 - sp) * dt, ti + (1 - 2 * sp) * dt, p))
    c.extend(_propagator_impl(terms, ti + dt, ti + (1 - sp) * dt, p))
    return c


def trotter_propagator(L, dims, bonds, sites=None, tspan=(0.0, 0.01), order=2, stepsize=0.01):
    """trotter_propagator(ham, tspan; order, stepsize) (tebd.jl:171-193) for a
    Hamiltonian given as bond terms {(i, i+1): h} and site terms {i: h} (fused index
    first site fastest), each a matrix or a function of t returning one; gates are
    exp(dt h(t)) with t the midpoint of their second-order step (tebd.jl:99-119)."""
    terms = _absorb_one_bodies(L, dims, bonds, sites or {})
    p = order // 2
    if 2 * p != order:
        raise ValueError("only even order supported.")
    ti, tf = tspan
    tdiff = tf - ti
    nsteps = int(round(abs(tdiff / stepsize))) or 1
    dt = tdiff / nsteps
    c = QuantumCircuit()
    for i in range(1, nsteps + 1):
        c.extend(_propagator_impl(terms, ti + i * dt, ti + (i - 1) * dt, p))
    return c


# ---------------------------------------------------------------- TEBD time stepping
def compute_step_size(t, dt):
    """compute_step_size (algorithms/timeevo.jl:3-9): n = round(|t / dt|) steps (at least
    one) of size t / n."""
    n = int(round(abs(t / dt))) or 1
    return n, t / n


class TEBDStepper:
    """TEBDStepper (algorithms/timeevo.jl:13-33): the span tspan cut into n steps of
    size stepsize (adjusted to divide it), the Trotter order and the truncation."""

    def __init__(self, stepsize, tspan=None, order=2, trunc=None):
        ti, tf = tspan if tspan is not None else (0.0, stepsize)
        self.n, self.stepsize = compute_step_size(tf - ti, stepsize)
        self.tspan = (ti, tf)
        self.order = int(order)
        self.trunc = trunc if trunc is not None else default_truncation()

    @property
    def delta(self):
        return self.tspan[1] - self.tspan[0]


class HomogeneousTEBDCache:
    """HomogeousTEBDCache (algorithms/timeevo.jl:88-99) for a constant Hamiltonian given
    as bond matrices {(i, i+1): h} and site matrices {i: h}: the circuit of n Trotter steps
    of size stepsize, fused once (fuse_gates of the repeated one-step circuit)."""

    def __init__(self, L, dims, bonds, sites, stepper):
        # the reference refuses a time-dependent Hamiltonian here (timeevo.jl:90)
        if any(callable(v) for v in list(dict(bonds).values()) + list(dict(sites).values())):
            raise ValueError("const hamiltonian expected.")
        one = trotter_propagator(L, dims, bonds, sites, tspan=(0.0, stepper.stepsize),
                                 order=stepper.order, stepsize=stepper.stepsize)
        self.circuit = fuse_gates(QuantumCircuit(list(one) * stepper.n))
        self.stepper = stepper


class InhomogeneousTEBDCache:
    """InhomogenousTEBDCache (algorithms/timeevo.jl:124-140) for a time-dependent
    Hamiltonian (bond and site terms may be functions of t): the fused Trotter circuit of
    the whole span tspan."""

    def __init__(self, L, dims, bonds, sites, stepper):
        self.circuit = fuse_gates(trotter_propagator(L, dims, bonds, sites,
                                                     tspan=stepper.tspan, order=stepper.order,
                                                     stepsize=stepper.stepsize))
        self.stepper = stepper


def make_step_(cache, psi, svd="gesvd"):
    """make_step! (algorithms/timeevo.jl:117-121): the cached circuit applied to psi with
    the stepper's truncation; returns the truncation error of every gate."""
    return apply_(cache.circuit, psi, trunc=cache.stepper.trunc, svd=svd)
