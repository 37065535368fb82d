"""CPU oracle of the learned density guess -- TEST INFRASTRUCTURE ONLY.

Only the tests (and smoke/bench checks) import this file; the library never calls it.  The learned
guess has no counterpart in the reference (which starts from the core Hamiltonian, RHF.hpp:205-211, or
reads PMATRIX.DAT, RHF.hpp:120-123), so this oracle pins itself: its FP64 gradient is checked against
central finite differences of its own loss (tests/test_guess_oracle.py), and the GPU's forward, loss and
gradients are checked against it (tests/test_guess_gpu.py).  It restates, in numpy and FP64:

  * features of an ordered atom pair (i, j): [onehot(elem i) | onehot(elem j) | exp(-((r - k d) / d)^2)],
    k < n_rbf, d = r_cut / (n_rbf - 1); self rows (i, i) have r = 0; elements in increasing Z;
  * the linear map from the network outputs of a row to density blocks, written as explicit matrices
    M_p (one per output p, in the library's output order):
      self row:      shell pairs a <= b of atom i: s-s (1), p-p isotropic delta_kl (1);
      pair row i->j: off-diagonal block over shells a of i, b of j: s-s (1), s-p e_l (1), p-s e_k (1),
                     p-p sigma e_k e_l and pi delta_kl - e_k e_l (2);
                     then on-site block of i over shell pairs a <= b: s-s (1), s-p e_k (1), p-p sigma, pi (2);
    every output scaled by f_c(r) = (cos(pi r / r_cut) + 1) / 2, P_ij = (B_ij + B_ji^T) / 2,
    P_ii = B_self + sum_j B_onsite(i; j); pairs with r >= r_cut are dropped;
  * the loss: mean over molecules of sum (P_pred - P_target)^2 over the full symmetric matrix;
  * the MLP: z_l = h_l W_l^T + b_l, h_{l+1} = silu(z_l), y = h_L W_L^T + b_L, and its backward pass.
With bf16=True the values the GPU rounds to BF16 are rounded the same way (inputs, weights,
activations h, the output gradient and the pre-activation gradients fed to the GEMMs).
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r.astype(np.uint32)).view(np.float32).astype(np.float64)


def _id(x):
    return np.asarray(x, np.float64)


def atom_shells(shell_l, shell_offset, shell_center, ncen):
    """Per centre: (first function, [(l, offset within the atom)])."""
    out = []
    for c in range(ncen):
        idx = [s for s in range(len(shell_l)) if shell_center[s] == c]
        f0 = shell_offset[idx[0]]
        out.append((f0, [(int(shell_l[s]), int(shell_offset[s] - f0)) for s in idx]))
    return out


def _nbf(sh):
    return sum((l + 1) * (l + 2) // 2 for l, _ in sh)


def self_mats(sh):
    n = _nbf(sh)
    mats = []
    for a in range(len(sh)):
        for b in range(a, len(sh)):
            (la, oa), (lb, ob) = sh[a], sh[b]
            if la == 0 and lb == 0:
                M = np.zeros((n, n))
                M[oa, ob] = M[ob, oa] = 1.0
                mats.append(M)
            elif la == 1 and lb == 1:
                M = np.zeros((n, n))
                for k in range(3):
                    M[oa + k, ob + k] = M[ob + k, oa + k] = 1.0
                mats.append(M)
    return mats


def pair_mats(shi, shj, e):
    """(off-diagonal matrices [nbf_i x nbf_j], on-site matrices [nbf_i x nbf_i]) of a row i -> j."""
    ni, nj = _nbf(shi), _nbf(shj)
    ee = np.outer(e, e)
    pi_ = np.eye(3) - ee
    off = []
    for la, oa in shi:
        for lb, ob in shj:
            if la == 0 and lb == 0:
                M = np.zeros((ni, nj)); M[oa, ob] = 1.0; off.append(M)
            elif la == 0 and lb == 1:
                M = np.zeros((ni, nj)); M[oa, ob:ob + 3] = e; off.append(M)
            elif la == 1 and lb == 0:
                M = np.zeros((ni, nj)); M[oa:oa + 3, ob] = e; off.append(M)
            else:
                M = np.zeros((ni, nj)); M[oa:oa + 3, ob:ob + 3] = ee; off.append(M)
                M = np.zeros((ni, nj)); M[oa:oa + 3, ob:ob + 3] = pi_; off.append(M)
    on = []
    for a in range(len(shi)):
        for b in range(a, len(shi)):
            (la, oa), (lb, ob) = shi[a], shi[b]
            if la == 0 and lb == 0:
                M = np.zeros((ni, ni)); M[oa, ob] = M[ob, oa] = 1.0; on.append(M)
            elif la != lb:
                os_, op = (oa, ob) if la == 0 else (ob, oa)
                M = np.zeros((ni, ni)); M[os_, op:op + 3] = e; M[op:op + 3, os_] = e; on.append(M)
            else:
                for blk in (ee, pi_):
                    M = np.zeros((ni, ni))
                    M[oa:oa + 3, ob:ob + 3] = blk
                    M[ob:ob + 3, oa:oa + 3] = blk.T
                    on.append(M)
    return off, on


class Molecule:
    """Rows, features and assembly matrices of one molecule."""

    def __init__(self, shell_l, shell_offset, shell_center, centers, charges, norb, elements, n_rbf=16,
                 r_cut=15.0):
        centers = np.asarray(centers, np.float64).reshape(-1, 3)
        ncen = len(centers)
        self.norb = norb
        sh = atom_shells(shell_l, shell_offset, shell_center, ncen)
        el = [elements.index(int(round(q))) for q in charges]
        E = len(elements)
        d = r_cut / (n_rbf - 1)
        self.rows = []  # (i, j, f0_i, f0_j, fc, mats_off, mats_on)
        feats = []

        def feat(ei, ej, r):
            x = np.zeros(2 * E + n_rbf)
            x[ei] = 1.0
            x[E + ej] = 1.0
            x[2 * E:] = np.exp(-(((r - d * np.arange(n_rbf)) / d) ** 2))
            return x

        for i in range(ncen):
            self.rows.append((i, i, sh[i][0], sh[i][0], 1.0, [], self_mats(sh[i][1])))
            feats.append(feat(el[i], el[i], 0.0))
        for i in range(ncen):
            for j in range(ncen):
                if i == j:
                    continue
                v = centers[j] - centers[i]
                r = float(np.linalg.norm(v))
                if r >= r_cut:
                    continue
                e = v / r
                off, on = pair_mats(sh[i][1], sh[j][1], e)
                fc = 0.5 * (np.cos(np.pi * r / r_cut) + 1.0)
                self.rows.append((i, j, sh[i][0], sh[j][0], fc, off, on))
                feats.append(feat(el[i], el[j], r))
        self.X = np.array(feats)

    def assemble(self, Y):
        """P from the network outputs Y [rows x n_out]."""
        P = np.zeros((self.norb, self.norb))
        for (i, j, fi, fj, fc, off, on), y in zip(self.rows, Y):
            k = 0
            for M in off:
                B = fc * y[k] * M
                P[fi:fi + B.shape[0], fj:fj + B.shape[1]] += 0.5 * B
                P[fj:fj + B.shape[1], fi:fi + B.shape[0]] += 0.5 * B.T
                k += 1
            for M in on:
                P[fi:fi + M.shape[0], fi:fi + M.shape[0]] += fc * y[k] * M
                k += 1
        return P

    def assemble_grad(self, G, n_out):
        """d/dY of sum(G * P(Y)) (the transpose of assemble)."""
        dY = np.zeros((len(self.rows), n_out))
        for r, (i, j, fi, fj, fc, off, on) in enumerate(self.rows):
            k = 0
            for M in off:
                blk = 0.5 * (G[fi:fi + M.shape[0], fj:fj + M.shape[1]] + G[fj:fj + M.shape[1], fi:fi + M.shape[0]].T)
                dY[r, k] = fc * np.sum(M * blk)
                k += 1
            for M in on:
                dY[r, k] = fc * np.sum(M * G[fi:fi + M.shape[0], fi:fi + M.shape[0]])
                k += 1
        return dY


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def unpack(p, n_in, hidden, layers, n_out):
    dims = [n_in] + [hidden] * layers + [n_out]
    out, k = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        W = np.asarray(p[k:k + din * dout], np.float64).reshape(dout, din)
        k += din * dout
        out.append((W, np.asarray(p[k:k + dout], np.float64)))
        k += dout
    return out


def pack(grads):
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def mlp_forward(params, X, bf=False):
    """Returns (Y, cache)."""
    rnd = bf16 if bf else _id
    h = rnd(X)
    cache = {"h": [h], "z": []}
    L = len(params) - 1
    for l, (W, b) in enumerate(params):
        z = h @ rnd(W).T + b
        if l == L:
            return z, cache
        cache["z"].append(z)
        h = rnd(silu(z))
        cache["h"].append(h)


def mlp_backward(params, cache, dY, bf=False):
    """Gradients [(dW, db)] of sum(dY * Y)."""
    rnd = bf16 if bf else _id
    L = len(params) - 1
    grads = [None] * (L + 1)
    g = rnd(dY)
    grads[L] = (g.T @ cache["h"][L], dY.sum(0))
    for l in range(L - 1, -1, -1):
        dz = (g @ rnd(params[l + 1][0])) * dsilu(cache["z"][l])
        gz = rnd(dz)
        grads[l] = (gz.T @ cache["h"][l], dz.sum(0))
        g = gz
    return grads


def loss_and_grad(params, mols, targets, n_out, bf=False):
    """Mean over molecules of sum (P - P*)^2 and its gradient (flat, host order)."""
    total = 0.0
    acc = None
    n = len(mols)
    for m, Pt in zip(mols, targets):
        Y, cache = mlp_forward(params, m.X, bf)
        Y = np.pad(Y, ((0, 0), (0, max(0, n_out - Y.shape[1]))))
        P = m.assemble(Y)
        D = P - Pt
        total += float(np.sum(D * D))
        dY = m.assemble_grad(2.0 * D / n, n_out)
        g = pack(mlp_backward(params, cache, dY, bf))
        acc = g if acc is None else acc + g
    return total / n, acc


def packed_to_full(pk, n):
    P = np.zeros((n, n))
    k = 0
    for i in range(n):
        for j in range(i + 1):
            P[i, j] = P[j, i] = pk[k]
            k += 1
    return P
