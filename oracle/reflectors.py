"""Q and P of the band reduction A = Q B P^T, rebuilt from the Householder
vectors that Blockbidiag! leaves in the tiles and the tau of every reflector.

TEST INFRASTRUCTURE ONLY: the orthogonality / backward-error check of the band
reduction.  It reads the layout of ``avs_blockbidiag_tau_dev`` (and of the
oracle's ``blockbidiag_keep``), which follows the tile factorisations of the
reference (paths inside evelyne-ringoot/Avocado-sandwich):

* QR half-step k (KAbasedSVD/src/tiledalgos.jl:21-24): GEQRT of tile (k, k)
  (QRkernels.jl:3-66; reflector l = e_l + the strictly lower column l of the
  tile, l < b - 1), then TSQRT of [R_kk; A_rk] for r = k+1 .. nt-1
  (QRkernels.jl:71-129; reflector l = e_l on the top tile + column l of tile
  (r, k) on the bottom one).  Each acts from the left: A <- H A.
* LQ half-step k (tiledalgos.jl:28-31, TiledMatrix.jl:85-113): the same on
  the adjoint of the row panel -- GELQT of tile (k, k+1) (reflector l = e_l +
  the strictly upper row l of the tile), then TSLQT of tile (k, c), c >= k+2
  (e_l on tile column k+1, row l of tile (k, c)).  Each acts from the right.

Every reflector is H = I - tau v v^T.  The reduction applies them in the order
above, so B = L_N ... L_1 A R_1 ... R_M and A = L_1 ... L_N B R_M ... R_1.
"""
import numpy as np


def _tile_factor(vs, taus, m):
    """Explicit m x m product H_0 H_1 ... of reflectors (columns of vs)."""
    q = np.eye(m)
    for l in range(vs.shape[1]):
        t = taus[l]
        if t == 0.0:
            continue
        v = vs[:, l]
        q -= t * np.outer(q @ v, v)
    return q


def tile_ops(a, tau_q, tau_p, b):
    """The tile factorisations of Blockbidiag! in application order: a list of
    (side, index array, m x m orthogonal factor), side 'L' (rows) or 'R'
    (columns); the factor is the product H_0 H_1 ... of the tile's reflectors."""
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    nt = n // b
    tq = np.asarray(tau_q, dtype=np.float64)
    tp = np.asarray(tau_p, dtype=np.float64)
    ops = []
    eye = np.eye(b)
    for k in range(nt):
        kb = np.arange(k * b, (k + 1) * b)
        # GEQRT of tile (k, k): unit lower V, reflectors 0 .. b-2
        t = a[k * b:(k + 1) * b, k * b:(k + 1) * b]
        v = np.tril(t, -1) + eye
        taus = tq[(k * nt + k) * b:(k * nt + k + 1) * b].copy()
        taus[b - 1] = 0.0
        ops.append(("L", kb, _tile_factor(v, taus, b)))
        for r in range(k + 1, nt):
            vb = a[r * b:(r + 1) * b, k * b:(k + 1) * b]
            v = np.vstack([eye, vb])
            taus = tq[(k * nt + r) * b:(k * nt + r + 1) * b]
            ops.append(("L", np.concatenate([kb, np.arange(r * b, (r + 1) * b)]), _tile_factor(v, taus, 2 * b)))
        if k == nt - 1:
            break
        k1 = np.arange((k + 1) * b, (k + 2) * b)
        # GELQT of tile (k, k+1): unit upper rows, reflectors 0 .. b-2
        t = a[k * b:(k + 1) * b, (k + 1) * b:(k + 2) * b]
        v = (np.triu(t, 1) + eye).T
        taus = tp[(k * nt + k + 1) * b:(k * nt + k + 2) * b].copy()
        taus[b - 1] = 0.0
        ops.append(("R", k1, _tile_factor(v, taus, b)))
        for c in range(k + 2, nt):
            vr = a[k * b:(k + 1) * b, c * b:(c + 1) * b].T
            v = np.vstack([eye, vr])
            taus = tp[(k * nt + c) * b:(k * nt + c + 1) * b]
            ops.append(("R", np.concatenate([k1, np.arange(c * b, (c + 1) * b)]), _tile_factor(v, taus, 2 * b)))
    return ops


def band_of(a, b):
    """Upper band 0 <= j - i <= b of a, zeros elsewhere (float64)."""
    a = np.asarray(a, dtype=np.float64)
    i, j = np.indices(a.shape)
    return np.where((j - i >= 0) & (j - i <= b), a, 0.0)


def rebuild(a, tau_q, tau_p, b):
    """(Q, P, B): Q = L_1 ... L_N and P = R_1 ... R_M as explicit float64
    matrices and the band B, so that A = Q B P^T."""
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    ops = tile_ops(a, tau_q, tau_p, b)
    q = np.eye(n)
    p = np.eye(n)
    for side, idx, f in ops:
        if side == "L":
            q[:, idx] = q[:, idx] @ f
        else:
            p[:, idx] = p[:, idx] @ f
    return q, p, band_of(a, b)


def checks(a_in, a_out, tau_q, tau_p, b):
    """Relative backward error ||A - Q B P^T||_F / ||A||_F and the losses of
    orthogonality ||Q^T Q - I||_F, ||P^T P - I||_F (float64 arithmetic)."""
    q, p, band = rebuild(a_out, tau_q, tau_p, b)
    a = np.asarray(a_in, dtype=np.float64)
    n = a.shape[0]
    back = float(np.linalg.norm(a - q @ band @ p.T) / np.linalg.norm(a))
    oq = float(np.linalg.norm(q.T @ q - np.eye(n)))
    op = float(np.linalg.norm(p.T @ p - np.eye(n)))
    return back, oq, op
