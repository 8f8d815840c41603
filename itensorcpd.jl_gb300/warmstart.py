"""Learned warm start for CP-ALS.

1. Sketch.  Y_n = T_(n) (Omega_b (.) Omega_a), an MTTKRP with seeded Gaussian test matrices
   (S columns per mode), computed by the engine's own MTTKRP; Q_n = orth(Y_n) spans the
   dominant column space of mode n.
2. Core.  G = T x_1 Q_0^T x_2 Q_1^T x_3 Q_2^T (S x S x S), again by the engine's MTTKRP:
   G_(0) = Q_0^T T_(0) (Q_2 (x) Q_1), the Kronecker product written as a Khatri-Rao product of
   column-repeated bases, S^2 columns in blocks the engine's rank allows.
3. Proposal.  Jennrich's simultaneous diagonalisation (Harshman 1970; Leurgans, Ross and
   Abel 1993) of the core: two random mode-3 contractions M1, M2 of G; the eigenvectors of
   M1 M2^+ and of M1^T M2^{+T} give the mode-1 and mode-2 coefficients, least squares the
   third.  It is exact for a noise-free core of rank R <= S with independent factors.
4. Teacher.  The batched solver (cpals_batch_*) runs ALS on the cores of many training
   tensors at once, from their proposals: one sweep gives the step D = P1 - P, convergence
   gives the core's own CP coefficients P*.  Sweeps on an S^3 core cost a fraction of a
   sweep on the full tensor, and the column order of P is kept.
5. Network.  A 3-layer MLP (BF16, FP32 accumulation, every product on the tensor cores,
   trained on the device by libcpals' own forward / backward / Adam kernels) maps the
   proposal and its one-sweep step of the three modes to the correction P* - P of each
   mode; the learned start is F_n = Q_n (P_n + s dP_n), columns normalised: it lies inside
   the sketched column range.  It costs one core sweep and one forward pass instead of the
   teacher's many sweeps.

Random-init ALS stays the fallback, and ALS decides when to stop: the warm start changes only
the starting point, ALS still runs to its convergence check, and a degenerate start (non-finite values
or a zero column) falls back to the reference's random start.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .synthetic import congruent_factor


# ---------------------------------------------------------------- the network

class WarmStartMLP:
    """Device MLP widths = (in, hidden1, hidden2, out) (cpals_mlp_*)."""

    def __init__(self, widths, device=0, params=None, seed=0):
        self.lib = L.load()
        self.widths = tuple(int(w) for w in widths)
        w = (C.c_int * 4)(*self.widths)
        h = C.c_void_p()
        L.check(self.lib.cpals_mlp_create(C.byref(h), int(device), w), "cpals_mlp_create")
        self.h = h
        self.n_params = int(self.lib.cpals_mlp_num_params(h))
        self.scale = 1.0  # step applied to the predicted correction (see calibrate)
        self.step_scale = 1.0  # unit of the one-sweep steps and corrections in the network's input and output
        self.step_gain = 0.0  # least-squares gain of the one-sweep step (see fit_step_gain)
        self.min_scale = 0.05
        self.set_params(self.init_params(np.random.default_rng(seed)) if params is None else params)

    def init_params(self, rng):
        """He-uniform weights, zero biases."""
        parts = []
        for l in range(3):
            n_in, n_out = self.widths[l], self.widths[l + 1]
            lim = np.sqrt(6.0 / n_in)
            parts.append(rng.uniform(-lim, lim, size=n_out * n_in).astype(np.float32))
            parts.append(np.zeros(n_out, dtype=np.float32))
        return np.concatenate(parts)

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpals_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _f(a):
        return a.ctypes.data_as(C.POINTER(C.c_float))

    def set_params(self, p):
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        L.check(self.lib.cpals_mlp_set_params(self.h, self._f(p)), "cpals_mlp_set_params")

    def get_params(self):
        p = np.empty(self.n_params, dtype=np.float32)
        L.check(self.lib.cpals_mlp_get_params(self.h, self._f(p)), "cpals_mlp_get_params")
        return p

    def forward(self, x):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        y = np.empty((x.shape[0], self.widths[3]), dtype=np.float32)
        L.check(self.lib.cpals_mlp_forward(self.h, self._f(x), x.shape[0], self._f(y)), "cpals_mlp_forward")
        return y

    def gradients(self, x, t):
        x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        t = np.ascontiguousarray(np.asarray(t, dtype=np.float32))
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_double()
        L.check(self.lib.cpals_mlp_gradients(self.h, self._f(x), self._f(t), x.shape[0], self._f(g),
                                             C.byref(loss)), "cpals_mlp_gradients")
        return loss.value, g

    def calibrate(self, X, T):
        """Least-squares step for the predicted correction on held-out pairs (X, T),
        scale = <P, T> / <P, P> clipped to [0, 1], and 0 below `min_scale`: a correction that
        does not generalise leaves the proposal untouched.  Returns the scale."""
        P = self.forward(X).astype(np.float64)
        T = np.asarray(T, dtype=np.float64)
        pp = float(np.sum(P * P))
        self.scale = float(np.clip(np.sum(P * T) / pp, 0.0, 1.0)) if pp > 0 else 0.0
        if self.scale < self.min_scale:
            self.scale = 0.0  # the correction does not generalise: the proposal is used as is
        return self.scale

    def train_stats(self, batch):
        """Device ms of the last training call's launches and the tensor-core flops of one step."""
        ms, fl = C.c_double(), C.c_double()
        L.check(self.lib.cpals_mlp_train_stats(self.h, int(batch), C.byref(ms), C.byref(fl)), "cpals_mlp_train_stats")
        return ms.value, fl.value

    def fit(self, X, T, epochs=30, batch=256, lr=1e-3, seed=0):
        """Adam on (X, T) held on the device; returns the per-step losses."""
        X = np.ascontiguousarray(np.asarray(X, dtype=np.float32))
        T = np.ascontiguousarray(np.asarray(T, dtype=np.float32))
        n = X.shape[0]
        L.check(self.lib.cpals_mlp_set_dataset(self.h, self._f(X), self._f(T), n), "cpals_mlp_set_dataset")
        rng = np.random.default_rng(seed)
        batch = min(batch, n)
        steps = n // batch
        losses = []
        self.fit_ms, self.fit_steps = 0.0, 0
        for _ in range(epochs):
            idx = rng.permutation(n)[: steps * batch].astype(np.int32)
            out = np.empty(steps)
            L.check(self.lib.cpals_mlp_train(self.h, idx.ctypes.data_as(C.POINTER(C.c_int)), steps, batch,
                                             float(lr), L.dptr(out)), "cpals_mlp_train")
            losses.extend(out.tolist())
            self.fit_ms += self.train_stats(batch)[0]
            self.fit_steps += steps
        return np.asarray(losses)


# ---------------------------------------------------------------- sketch and features

def gaussian_test_matrices(dims, S, seed):
    """Seeded Gaussian test matrices Omega_m (I_m x S), entries N(0, 1/I_m)."""
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((d, S)) / np.sqrt(d) for d in dims]


def sketch(engine, omegas):
    """Y_n = T_(n) (Omega_b (.) Omega_a) for every mode (the engine's MTTKRP with Gaussian factors)."""
    engine.set_factors(omegas, np.ones(omegas[0].shape[1]))
    return [engine.mttkrp(n) for n in range(len(omegas))]


def sketch_bases(Ys):
    """Orthonormal bases Q_n of the sketches and their normalised summaries Z_n = Q_n^T Y_n."""
    Qs, Zs = [], []
    for Y in Ys:
        Q, Z = np.linalg.qr(Y)
        s = np.sign(np.diag(Z))
        s[s == 0] = 1.0
        Q = Q * s[None, :]
        Z = Z * s[:, None]
        Qs.append(Q)
        Zs.append(Z / max(np.linalg.norm(Z), 1e-300))
    return Qs, Zs


def features(props, steps, step_scale=1.0):
    """Network input of each mode n of each tensor: [P_n, D_n / step_scale] of its own mode,
    then of the other modes in mode order (P the proposal's coefficients, D the one-sweep
    step), as rows of FP32."""
    rows = []
    for P, D in zip(props, steps):
        N = len(P)
        for n in range(N):
            parts = []
            for m in [n] + [m for m in range(N) if m != n]:
                parts += [np.asarray(P[m]).ravel(), np.asarray(D[m]).ravel() / step_scale]
            rows.append(np.concatenate(parts))
    return np.asarray(rows, dtype=np.float32)


def targets(props, solved, step_scale=1.0):
    """Training targets: the correction P*_n - P_n of every mode (in units of step_scale)."""
    return np.asarray([((np.asarray(C) - np.asarray(P)) / step_scale).ravel()
                       for Ps, Cs in zip(props, solved) for P, C in zip(Ps, Cs)], dtype=np.float32)


def core_als(be, cores, starts, max_iter, tol=0.0):
    """ALS on S^3 cores with the batched solver `be` (a BatchEngine sized for these cores),
    from coefficient starts with unit columns.  Returns the coefficients (unit columns, each
    column signed like its start) and the sweeps each core ran."""
    R = starts[0][0].shape[1]
    be.set_norms([max(float(np.linalg.norm(G)), 1e-300) for G in cores])
    be.set_tensors([np.asarray(G, dtype=np.float32) for G in cores])
    be.set_factors(starts, [np.ones(R)] * len(cores))
    sweeps, _, _, _ = be.optimize(tol=tol, max_iter=max_iter)
    out = []
    for (F, _), P in zip(be.get_factors(), starts):
        C = []
        for Fn, Pn in zip(F, P):
            sg = np.sign(np.sum(Fn * Pn, axis=0))
            sg[sg == 0] = 1.0
            C.append(Fn * sg[None, :])
        out.append(C)
    return out, sweeps


def core(core_engine, Qs):
    """G (S x S x S) = T x_n Q_n^T from mode-0 MTTKRPs of an engine whose rank is a divisor
    of S^2: column c = j S + i of the Khatri-Rao factors is Q_1(:, i) and Q_2(:, j)."""
    S = Qs[0].shape[1]
    blk = core_engine.rank
    M = np.empty((Qs[0].shape[0], S * S))
    cols = np.arange(S * S)
    for c0 in range(0, S * S, blk):
        c = cols[c0:c0 + blk]
        F1 = Qs[1][:, c % S]
        F2 = Qs[2][:, c // S]
        F0 = np.zeros((Qs[0].shape[0], blk))
        core_engine.set_factors([F0, F1, F2], np.ones(blk))
        M[:, c0:c0 + blk] = core_engine.mttkrp(0)
    G0 = Qs[0].T @ M  # S x S^2, column i1 + S i2
    return np.reshape(G0, (S, S, S), order="F")


def jennrich(G, R, rng):
    """CP proposal of the core by simultaneous diagonalisation; unit columns, components
    ordered by decreasing |eigenvalue|.  A complex-conjugate pair of eigenvalues among the R
    kept gives the real and imaginary parts of its eigenvector as two columns (the real
    invariant subspace of the pair), so no two columns repeat."""
    S = G.shape[0]
    x, y = rng.standard_normal(S), rng.standard_normal(S)
    M1 = np.tensordot(G, x, axes=([2], [0]))
    M2 = np.tensordot(G, y, axes=([2], [0]))
    ev, V = np.linalg.eig(M1 @ np.linalg.pinv(M2))
    order = list(np.argsort(-np.abs(ev))[:R])
    ev2, V2 = np.linalg.eig(M1.T @ np.linalg.pinv(M2.T))
    A = np.empty((S, R))
    B = np.empty((S, R))
    done = set()
    for k, j in enumerate(order):
        if k in done:
            continue
        e = ev[j]
        vb = V2[:, np.argmin(np.abs(ev2 - e))]
        A[:, k], B[:, k] = np.real(V[:, j]), np.real(vb)
        done.add(k)
        if abs(e.imag) > 1e-12 * max(abs(e), 1e-300):
            # the conjugate partner, if kept: the imaginary parts
            part = [q for q in range(k + 1, R) if q not in done and abs(ev[order[q]] - np.conj(e)) <= 1e-9 * abs(e)]
            if part:
                q = part[0]
                A[:, q], B[:, q] = np.imag(V[:, j]), np.imag(vb)
                done.add(q)
    A = A / np.maximum(np.linalg.norm(A, axis=0), 1e-300)
    B = B / np.maximum(np.linalg.norm(B, axis=0), 1e-300)
    K = (B[:, None, :] * A[None, :, :]).reshape(S * S, R)  # column r = B(:, r) (x) A(:, r)
    G2 = np.reshape(np.moveaxis(G, 2, 0), (S, S * S), order="F")  # mode-3 unfolding, i1 + S i2
    C = np.linalg.lstsq(K, G2.T, rcond=None)[0].T
    C = C / np.maximum(np.linalg.norm(C, axis=0), 1e-300)
    return [A, B, C]
def proposal_factors(Qs, proposal):
    """The start without the network: F_n = Q_n C_n from the proposal."""
    return _lift(Qs, proposal)


def fit_step_gain(X, Y, SR):
    """Least-squares gain a of the one-sweep step (the second S*R block of each feature row)
    as a predictor of the target rows: the linear part of the correction, which the network
    then refines."""
    D = X[:, SR:2 * SR].astype(np.float64)
    return float(np.sum(D * Y) / max(np.sum(D * D), 1e-300))


def residual_targets(X, Y, SR, gain):
    """What the network learns: the target less the gain times the step."""
    return (Y - gain * X[:, SR:2 * SR]).astype(np.float32)


def learned_coefficients(mlp, props, steps):
    """P + a D + s dP for each tensor: the step's least-squares gain a (mlp.step_gain) plus the
    network's correction of what is left, times its calibrated step s."""
    X = features(props, steps, mlp.step_scale)
    SR = props[0][0].size
    D = (mlp.step_gain * X[:, SR:2 * SR] + mlp.forward(X) * mlp.scale) * mlp.step_scale
    out, k = [], 0
    for P in props:
        C = []
        for Pn in P:
            C.append(Pn + D[k].astype(np.float64).reshape(Pn.shape))
            k += 1
        out.append(C)
    return out


def warm_factors(mlp, Qs, proposal, step):
    """The learned start of one tensor: F_n = Q_n (P_n + s dP_n); None if degenerate."""
    return _lift(Qs, learned_coefficients(mlp, [proposal], [step])[0])


def lift(Qs, Cs):
    """F_n = Q_n C_n with unit columns; None if degenerate."""
    return _lift(Qs, Cs)


def _lift(Qs, Cs):
    F = []
    for Q, Cn in zip(Qs, Cs):
        Fn = Q @ Cn
        nrm = np.linalg.norm(Fn, axis=0)
        if not np.all(np.isfinite(Fn)) or np.any(nrm < 1e-8):
            return None
        F.append(Fn / nrm)
    return F


def subspace_factors(Qs, R, rng):
    """The same start without the network: random coefficients inside the sketched range."""
    F = []
    for Q in Qs:
        Fn = Q @ rng.standard_normal((Q.shape[1], R))
        F.append(Fn / np.linalg.norm(Fn, axis=0))
    return F


# ---------------------------------------------------------------- synthetic tensors on the device

def synth_device(dims, rank, congruence, snr_db, rng, out_ptr, device=0, seed=None):
    """Low-rank-plus-noise tensor generated on the device into the FP32 buffer at out_ptr
    (column-major); factors are congruent (synthetic.congruent_factor), weights U[1, 10]."""
    lib = L.load()
    facs = [congruent_factor(d, rank, congruence, rng) for d in dims]
    w = rng.uniform(1.0, 10.0, size=rank)
    Fc = np.ascontiguousarray(np.concatenate([np.asarray(f, dtype=np.float64).ravel(order="F") for f in facs]))
    d = np.asarray(dims, dtype=np.int64)
    seed = int(rng.integers(0, 2**62)) if seed is None else int(seed)
    L.check(lib.cpals_synth_lowrank(int(device), len(dims), L.i64ptr(d), int(rank), L.dptr(Fc),
                                    L.dptr(np.ascontiguousarray(w)), float(snr_db), seed, C.c_void_p(int(out_ptr))),
            "cpals_synth_lowrank")
    return facs, w


def sweeps_to_fit(traj, target):
    """First sweep (1-based) whose fit reaches target, or None."""
    hit = np.nonzero(np.asarray(traj) >= target)[0]
    return int(hit[0]) + 1 if hit.size else None
