"""CPU restatement of tetragono's DirectSampling with its truncating contractions (test infrastructure
only; the checker for a direct sampler, never the product).  Dense float64 tensors without symmetry
(real, so every bra tensor equals its ket).

* ``double_down_line``: ``DoubleLayerAuxiliaries._two_line_to_one_line`` for the down-to-up family
  (tetragono/tetragono/auxiliaries/double_layer_auxiliaries.py:387-392, 416-496): the ket row is absorbed
  into the boundary line, QR sweep left to right, truncating SVD sweep right to left (singular values
  divided by their sum when ``normalize``); then the bra row, contracting the physical legs, and the
  same two sweeps.
* ``lr_step``: ``ThreeLineAuxiliaries._two_line_to_one_line`` (three_line_auxiliaries.py:68-117): the
  five-layer column (up boundary ket, row ket, double-layer down boundary, row bra, up boundary bra)
  absorbed into a left environment [rn0, rn1, big, rc1, rc0], the up boundary tensors split by QR, the
  ket and then the bra bond of ``big`` truncated by SVD; the right environment is the same step on the
  mirrored lattice.
* ``hole``: ``ThreeLineAuxiliaries.hole`` (three_line_auxiliaries.py:133-162): rho(I, O) of one site.
* ``DirectSampler``: ``DirectSampling.__call__`` (tetragono/tetragono/sampling_lattice/sampling.py:276-371):
  row by row, the up boundary is the single-layer boundary of the rows already sampled
  (``Configuration._up_to_down_site``, compressed as in peps_oracle.compress), the down boundary the
  double-layer one of the rows below; site by site, rho = diag(hole), clipped at 0, raised to alpha,
  normalised; one uniform_real(0, 1) draw and the cumulative ``_choice`` rule pick the index; the site
  is replaced by its projection for the rest of the row.
"""
import numpy as np

from .peps_oracle import Environment
from .rng import uniform_real01


def _sweeps(S, cut, normalize):
    """QR sweep left to right, then truncating SVD sweep right to left, over sites (A, open, B)."""
    n = len(S)
    for i in range(n - 1):
        A, o, B = S[i].shape
        q, r = np.linalg.qr(S[i].reshape(A * o, B))
        k = q.shape[1]
        S[i] = q.reshape(A, o, k)
        b, o2, c = S[i + 1].shape
        S[i + 1] = (r @ S[i + 1].reshape(b, o2 * c)).reshape(k, o2, c)
    for i in reversed(range(1, n)):
        A, o, B = S[i].shape
        u, s, vh = np.linalg.svd(S[i].reshape(A, o * B), full_matrices=False)
        k = min(cut, len(s))
        u, s, vh = u[:, :k], s[:k], vh[:k]
        if normalize:
            s = s / np.abs(s).sum()
        S[i] = vh.reshape(k, o, B)
        a, o1, b = S[i - 1].shape
        S[i - 1] = (S[i - 1].reshape(a * o1, b) @ (u * s)).reshape(a, o1, k)
    return S


def double_down_line(line, row, cut, normalize=True):
    """New down boundary (L, R, UN, UC) per site from ``line`` (L, R, UN, UC) and row sites (p, u, d, l, r)."""
    n = len(row)
    S = []
    for i in range(n):
        t = np.einsum("abxc,puxlr->alcupbr", line[i], row[i])       # line.UN x site.D
        a, l, c, u, p, b, r = t.shape
        S.append(t.reshape(a * l, c * u * p, b * r))
    S = _sweeps(S, cut, normalize)
    S2 = []
    for i in range(n):
        A, _, B = S[i].shape
        c, (p, u) = line[i].shape[3], row[i].shape[:2]
        t = np.einsum("acupb,pyclr->aluybr", S[i].reshape(A, c, u, p, B), row[i])   # UC x bra.D, P x P
        a, l, uu, yy, b, r = t.shape
        S2.append(t.reshape(a * l, uu * yy, b * r))
    S2 = _sweeps(S2, cut, normalize)
    return [S2[i].reshape(S2[i].shape[0], row[i].shape[1], row[i].shape[1], S2[i].shape[2]).transpose(0, 3, 1, 2)
            for i in range(n)]


ONES = (np.ones((1, 1)), np.ones((1, 1, 1)), np.ones((1, 1, 1)), np.ones((1, 1, 1)), np.ones((1, 1)))


def lr_step(env, col, cut):
    """env: rn0 (R, D), rn1 (U, R, D), big (UN, UC, R), rc1 (U, R, D), rc0 (R, D); col: n0 (L, D, R),
    n1 (p, u, d, l, r), t2 (L, R, UN, UC), c1 = n1, c0 = n0."""
    rn0, rn1, big, rc1, rc0 = env
    n0, n1, t2, c1, c0 = col

    def half(x0, r0, r1, x1):
        L, D0, R = x0.shape
        q, rr = np.linalg.qr(x0.transpose(2, 0, 1).reshape(R, L * D0))   # Q keeps R: (R, k)
        nr = rr.reshape(q.shape[1], L, D0)                                # (U = k, L, D0)
        t = np.einsum("kLd,Le->kde", nr, r0)                              # nr.L x rn0.R
        t = np.einsum("kdu,uRe->kdRe", t, r1)                             # rn0.D x rn1.U
        return q, np.einsum("kdRe,pdzRr->kerzp", t, x1)                   # D0 x n1.U, rn1.R x n1.L

    q_n, n12 = half(n0, rn0, rn1, n1)
    q_c, c12 = half(c0, rc0, rc1, c1)
    b = np.einsum("kerzp,eyR->krzpyR", n12, big)                          # rn1.D x big.UN
    b = np.einsum("krzpyR,RSzw->krpySw", b, t2)                           # n1.D x t2.UN, big.R x t2.L
    b = np.einsum("krpySw,jyswp->krSjs", b, c12)                          # bra side and the physical legs
    k, r, R2, kk, rr = b.shape
    u, sv, vh = np.linalg.svd(b.reshape(k * r, R2 * kk * rr), full_matrices=False)
    K = min(cut, len(sv))
    rn1_new = u[:, :K].reshape(k, r, K)
    b = (sv[:K, None] * vh[:K]).reshape(K, R2, kk, rr)
    u, sv, vh = np.linalg.svd(b.transpose(2, 3, 0, 1).reshape(kk * rr, K * R2), full_matrices=False)
    K2 = min(cut, len(sv))
    rc1_new = u[:, :K2].reshape(kk, rr, K2)
    big_new = (sv[:K2, None] * vh[:K2]).reshape(K2, K, R2).transpose(1, 0, 2)
    return (q_n, rn1_new, big_new, rc1_new, q_c)


def _mirror(col):
    n0, n1, t2, c1, c0 = col
    return (n0.transpose(2, 1, 0), n1.transpose(0, 1, 2, 4, 3), t2.transpose(1, 0, 2, 3),
            c1.transpose(0, 1, 2, 4, 3), c0.transpose(2, 1, 0))


def hole(left, right, col):
    """rho(I, O) of the column's site; ``right`` is a right environment in mirrored form."""
    rn0L, rn1L, bigL, rc1L, rc0L = left
    rn0R, rn1R, bigR, rc1R, rc0R = right
    n0, n1, t2, c1, c0 = col
    r = np.einsum("xa,xdR->adR", rn0L, n0)
    r = np.einsum("adR,Rc->adc", r, rn0R)
    r = np.einsum("adc,aRe->dcRe", r, rn1L)
    r = np.einsum("dcRe,odzRx->cezxo", r, n1)
    r = np.einsum("cezxo,cxf->ezof", r, rn1R)
    r = np.einsum("ezof,eyR->zofyR", r, bigL)
    r = np.einsum("zofyR,RSzw->ofySw", r, t2)
    r = np.einsum("ofySw,fvS->oywv", r, bigR)
    r = np.einsum("oywv,gRy->owvgR", r, rc1L)
    r = np.einsum("owvgR,ihwRx->ovgxhi", r, c1)
    r = np.einsum("ovgxhi,txv->oghit", r, rc1R)
    r = np.einsum("oghit,Rg->ohitR", r, rc0L)
    r = np.einsum("ohitR,RhX->oitX", r, c0)
    return np.einsum("oitX,Xt->io", r, rc0R)


class DirectSampler:
    """One ``DirectSampling`` process: ``peps`` (DensePEPS, cut = the single-layer cut), the engine of
    its draws, the double-layer cut and alpha."""

    def __init__(self, peps, engine, double_cut, alpha=1.0):
        self.peps, self.engine, self.alpha = peps, engine, alpha
        L1, L2 = peps.L1, peps.L2
        self.down = {L1: [np.ones((1, 1, 1, 1)) for _ in range(L2)]}
        for l1 in reversed(range(L1)):
            self.down[l1] = double_down_line(self.down[l1 + 1], [peps.A[l1][l2] for l2 in range(L2)], double_cut)

    def __call__(self):
        peps, cut = self.peps, self.peps.cut
        L1, L2 = peps.L1, peps.L2
        conf = np.zeros((L1, L2), dtype=np.int64)
        possibility = 1.0
        for l1 in range(L1):
            up = [np.ones((1, 1, 1)) for _ in range(L2)] if l1 == 0 else Environment(peps, conf).up(l1 - 1)
            row = [peps.A[l1][l2] for l2 in range(L2)]
            for l2 in range(L2):
                cols = [(up[c], row[c], self.down[l1 + 1][c], row[c], up[c]) for c in range(L2)]
                left = ONES
                for c in range(l2):
                    left = lr_step(left, cols[c], cut)
                right = ONES
                for c in reversed(range(l2 + 1, L2)):
                    right = lr_step(right, _mirror(cols[c]), cut)
                rho = np.maximum(np.diagonal(hole(left, right, cols[l2])), 0.0)
                if rho.sum() == 0:
                    raise NotImplementedError("zero marginal: the reference redraws the whole sample")
                rho = rho**self.alpha
                rho = rho / rho.sum()
                p = uniform_real01(self.engine)
                choice = len(rho) - 1
                for i, r in enumerate(rho):
                    p -= r
                    if p < 0:
                        choice = i
                        break
                possibility *= rho[choice]
                conf[l1, l2] = choice
                row[l2] = row[l2][choice:choice + 1]
        return possibility, conf
