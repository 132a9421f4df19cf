/*
 * CPU restatement of the reference tiled-SVD hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle: it is included twice by oracle.c, once with
 * OT = float (suffix _s) and once with OT = double (suffix _d).  Nothing in the
 * product library links it; only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it, as the parity reference.
 *
 * What it restates (paths are inside evelyne-ringoot/Avocado-sandwich):
 *   - GEQRT tile kernel            KAbasedSVD/src/QRkernels.jl:3-66
 *   - TSQRT tile kernel            KAbasedSVD/src/QRkernels.jl:71-129
 *   - apply Q / Q^T (single)       KAbasedSVD/src/QRkernels.jl:131-161
 *   - apply Q / Q^T (triangle-on-square pair)  KAbasedSVD/src/QRkernels.jl:165-197
 *   - tile views, LQ = QR on the adjoint       KAbasedSVD/src/TiledMatrix.jl:77-113
 *   - GE2BND schedule Blockbidiag!             KAbasedSVD/src/tiledalgos.jl:17-59
 *   - band -> bidiagonal (multi-stage halving) KAbasedSVD/src/bulgechasing.jl:1-42
 *
 * The arithmetic follows the reference formulas literally (element type OT,
 * the same nu / tau expressions), with one documented divergence: when a
 * column is exactly zero (s == 0 and alpha == 0) the reference divides 0/0
 * (sign(0) == 0 in Julia); here the reflector becomes the identity (tau = 0),
 * which is LAPACK's convention.  The s == 0, alpha != 0 case keeps the
 * reference's tau = 2 (a sign flip of the pivot row).
 *
 * Strided views model Julia's adjoint views: element (i, j) of a view lives at
 * p[i * rs + j * cs]; a normal column-major view has rs = 1, cs = ld, and its
 * adjoint swaps the two strides.
 */

#define OSUF2(a, b) a##b
#define OSUF1(a, b) OSUF2(a, b)
#define OSUF(name) OSUF1(name, OT_SUFFIX)

typedef struct {
    OT *p;
    int64_t rs, cs;
} OSUF(oview);

static inline OT *OSUF(oel)(OSUF(oview) v, int64_t i, int64_t j) {
    return v.p + i * v.rs + j * v.cs;
}

static inline OSUF(oview) OSUF(ov_cm)(OT *p, int64_t ld) {
    OSUF(oview) v = {p, 1, ld};
    return v;
}

static inline OSUF(oview) OSUF(ov_adj)(OSUF(oview) v) {
    OSUF(oview) w = {v.p, v.cs, v.rs};
    return w;
}

static inline OSUF(oview) OSUF(ov_sub)(OSUF(oview) v, int64_t i0, int64_t j0) {
    OSUF(oview) w = {v.p + i0 * v.rs + j0 * v.cs, v.rs, v.cs};
    return w;
}

/* Julia sign(): the zero case is handled by the caller (see header). */
static inline OT OSUF(osign)(OT x) { return x < (OT)0 ? (OT)-1 : (OT)1; }

/*
 * GEQRT on one b x b tile (QRkernels.jl:3-66, QR_unsafe_kernel!).
 * R in the upper triangle, V (unit diagonal implied) strictly below, tau[0..b-2];
 * tau[b-1] is left untouched (the reference loops iter = 1:N-1).
 */
void OSUF(oracle_geqrt_v)(OSUF(oview) A, int b, OT *tau) {
    OT *w = (OT *)malloc(sizeof(OT) * (size_t)b);
    for (int it = 0; it < b - 1; ++it) {
        OT s = 0;
        for (int t = it + 1; t < b; ++t) {
            OT x = *OSUF(oel)(A, t, it);
            s += x * x;
        }
        OT alpha = *OSUF(oel)(A, it, it);
        OT n1 = (OT)sqrt((double)(s + alpha * alpha));
        OT nu = alpha + OSUF(osign)(alpha) * n1;
        if (nu == (OT)0) { /* zero column: identity reflector */
            tau[it] = 0;
            for (int t = it + 1; t < b; ++t) *OSUF(oel)(A, t, it) = 0;
            continue;
        }
        OT n2 = (OT)sqrt((double)(s + nu * nu));
        OT q = nu / n2;
        OT tv = 2 * (q * q);
        tau[it] = tv;
        OT taucorr = tv / nu;
        for (int j = it; j < b; ++j) {
            OT acc = nu * *OSUF(oel)(A, it, j);
            for (int t = it + 1; t < b; ++t) acc += *OSUF(oel)(A, t, it) * *OSUF(oel)(A, t, j);
            w[j] = acc;
        }
        for (int j = it + 1; j < b; ++j) *OSUF(oel)(A, it, j) -= taucorr * w[j];
        for (int t = it + 1; t < b; ++t) {
            OT c = *OSUF(oel)(A, t, it) * taucorr / nu;
            for (int j = it + 1; j < b; ++j) *OSUF(oel)(A, t, j) -= c * w[j];
            *OSUF(oel)(A, t, it) = c / taucorr;
        }
        *OSUF(oel)(A, it, it) -= w[it] * taucorr;
    }
    free(w);
}

void OSUF(oracle_geqrt)(OT *a, int64_t lda, int b, OT *tau) {
    OSUF(oview) A = OSUF(ov_cm)(a, lda);
    OSUF(oracle_geqrt_v)(A, b, tau);
}

/*
 * TSQRT on the pair [R; B] (QRkernels.jl:71-129, QR_unsafe_kernel2!): R is the
 * b x b upper triangle of the top tile (its strictly-lower part is not read),
 * B the full b x b bottom tile, which receives V; tau[0..b-1].
 */
void OSUF(oracle_tsqrt_v)(OSUF(oview) R, OSUF(oview) B, int b, OT *tau) {
    OT *w = (OT *)malloc(sizeof(OT) * (size_t)b);
    for (int it = 0; it < b; ++it) {
        OT s = 0;
        for (int t = 0; t < b; ++t) {
            OT x = *OSUF(oel)(B, t, it);
            s += x * x;
        }
        OT alpha = *OSUF(oel)(R, it, it);
        OT n1 = (OT)sqrt((double)(s + alpha * alpha));
        OT nu = alpha + OSUF(osign)(alpha) * n1;
        if (nu == (OT)0) {
            tau[it] = 0;
            for (int t = 0; t < b; ++t) *OSUF(oel)(B, t, it) = 0;
            continue;
        }
        OT n2 = (OT)sqrt((double)(s + nu * nu));
        OT q = nu / n2;
        OT tv = 2 * (q * q);
        tau[it] = tv;
        OT taucorr = tv / nu;
        for (int j = it; j < b; ++j) {
            OT acc = nu * *OSUF(oel)(R, it, j);
            for (int t = 0; t < b; ++t) acc += *OSUF(oel)(B, t, it) * *OSUF(oel)(B, t, j);
            w[j] = acc;
        }
        for (int j = it; j < b; ++j) *OSUF(oel)(R, it, j) -= w[j] * taucorr;
        for (int t = 0; t < b; ++t) {
            OT c = *OSUF(oel)(B, t, it) / nu * taucorr;
            for (int j = it + 1; j < b; ++j) *OSUF(oel)(B, t, j) -= c * w[j];
            *OSUF(oel)(B, t, it) = c / taucorr;
        }
    }
    free(w);
}

void OSUF(oracle_tsqrt)(OT *r, int64_t ldr, OT *bt, int64_t ldb, int b, OT *tau) {
    OSUF(oracle_tsqrt_v)(OSUF(ov_cm)(r, ldr), OSUF(ov_cm)(bt, ldb), b, tau);
}

/*
 * Apply the GEQRT reflectors to a b x ncols block (QRkernels.jl:131-161):
 * trans != 0 applies Q^T (k = 1..b-1), trans == 0 applies Q (k = b-1..1).
 * Columns are independent, as in the reference's one-work-group-per-column
 * launch; OpenMP spreads them over the host cores.
 */
void OSUF(oracle_apply1_v)(OSUF(oview) Bm, int64_t ncols, OSUF(oview) V, const OT *tau, int b, int trans) {
#pragma omp parallel for schedule(static) if (ncols >= 64)
    for (int64_t i = 0; i < ncols; ++i) {
        for (int kk = 0; kk < b - 1; ++kk) {
            int k = trans ? kk : (b - 2 - kk);
            OT t = *OSUF(oel)(Bm, k, i);
            for (int j = k + 1; j < b; ++j) t += *OSUF(oel)(V, j, k) * *OSUF(oel)(Bm, j, i);
            t = t * tau[k];
            for (int j = k + 1; j < b; ++j) *OSUF(oel)(Bm, j, i) -= t * *OSUF(oel)(V, j, k);
            *OSUF(oel)(Bm, k, i) -= t;
        }
    }
}

void OSUF(oracle_apply1)(OT *bm, int64_t ldb, int64_t ncols, const OT *v, int64_t ldv, const OT *tau, int b,
                         int trans) {
    OSUF(oracle_apply1_v)(OSUF(ov_cm)(bm, ldb), ncols, OSUF(ov_cm)((OT *)v, ldv), tau, b, trans);
}

/*
 * Apply the TSQRT reflectors to the pair [A; B], each b x ncols
 * (QRkernels.jl:165-197); trans != 0 applies Q^T (k = 1..b), else Q (k = b..1).
 */
void OSUF(oracle_apply2_v)(OSUF(oview) Am, OSUF(oview) Bm, int64_t ncols, OSUF(oview) V, const OT *tau, int b,
                           int trans) {
#pragma omp parallel for schedule(static) if (ncols >= 64)
    for (int64_t i = 0; i < ncols; ++i) {
        for (int kk = 0; kk < b; ++kk) {
            int k = trans ? kk : (b - 1 - kk);
            OT t = *OSUF(oel)(Am, k, i);
            for (int j = 0; j < b; ++j) t += *OSUF(oel)(V, j, k) * *OSUF(oel)(Bm, j, i);
            t = t * tau[k];
            *OSUF(oel)(Am, k, i) -= t;
            for (int j = 0; j < b; ++j) *OSUF(oel)(Bm, j, i) -= t * *OSUF(oel)(V, j, k);
        }
    }
}

void OSUF(oracle_apply2)(OT *am, int64_t lda, OT *bm, int64_t ldb, int64_t ncols, const OT *v, int64_t ldv,
                         const OT *tau, int b, int trans) {
    OSUF(oracle_apply2_v)(OSUF(ov_cm)(am, lda), OSUF(ov_cm)(bm, ldb), ncols, OSUF(ov_cm)((OT *)v, ldv), tau, b,
                          trans);
}

/*
 * GE2BND: Blockbidiag! (tiledalgos.jl:17-59) over the tile views of
 * TiledMatrix.jl:77-113.  keep == 0: on return a (n x n, column-major, lda)
 * holds the upper band 0 <= j - i <= b with exact zeros elsewhere
 * (triu!/tril!/.= 0), as in the reference.  keep != 0: the Householder vectors
 * stay where the factorisations leave them (nothing later reads those
 * entries, so the band is the same), and the tau of every tile factorisation
 * go to tq / tp (nt * nt * b each; QR half-step k, tile row r at (k*nt + r)*b;
 * LQ half-step k, tile column c at (k*nt + c)*b), where the reference's Tau
 * grid keeps only the last one written to each slot.
 */
static void OSUF(blockbidiag_impl)(OT *a, int64_t n, int64_t lda, int b, int keep, OT *tq, OT *tp) {
    int64_t nt = n / b;
    OSUF(oview) A = OSUF(ov_cm)(a, lda);
    OT *tau = (OT *)calloc((size_t)b, sizeof(OT));
#define TILE(r, c) OSUF(ov_sub)(A, (int64_t)(r) * b, (int64_t)(c) * b)
#define KEEP_TAU(dst, k, t)                                                            \
    do {                                                                               \
        if (keep) memcpy((dst) + ((size_t)(k) * nt + (t)) * b, tau, sizeof(OT) * b); \
    } while (0)
    for (int64_t k = 0; k < nt; ++k) {
        /* QRandmulQt1!: QR1!, Qtapply1_par!, triu! */
        memset(tau, 0, sizeof(OT) * b);
        OSUF(oracle_geqrt_v)(TILE(k, k), b, tau);
        KEEP_TAU(tq, k, k);
        OSUF(oracle_apply1_v)(TILE(k, k + 1), (nt - k - 1) * b, TILE(k, k), tau, b, 1);
        if (!keep)
            for (int i = 0; i < b; ++i)
                for (int t = i + 1; t < b; ++t) *OSUF(oel)(TILE(k, k), t, i) = 0;
        /* QRandmulQt2!: QR2!, Qtapply2_par!, tile .= 0 */
        for (int64_t row = k + 1; row < nt; ++row) {
            OSUF(oracle_tsqrt_v)(TILE(k, k), TILE(row, k), b, tau);
            KEEP_TAU(tq, k, row);
            OSUF(oracle_apply2_v)(TILE(k, k + 1), TILE(row, k + 1), (nt - k - 1) * b, TILE(row, k), tau, b, 1);
            if (!keep)
                for (int j = 0; j < b; ++j)
                    for (int t = 0; t < b; ++t) *OSUF(oel)(TILE(row, k), t, j) = 0;
        }
        if (k == nt - 1) break;
        /* LQandmulQt1!: LQ1! = QR1! on tile(k,k+1)', LQtapply1_par! on the
         * adjoint of the column panel below, tril! */
        memset(tau, 0, sizeof(OT) * b);
        OSUF(oracle_geqrt_v)(OSUF(ov_adj)(TILE(k, k + 1)), b, tau);
        KEEP_TAU(tp, k, k + 1);
        OSUF(oracle_apply1_v)(OSUF(ov_adj)(TILE(k + 1, k + 1)), (nt - k - 1) * b, OSUF(ov_adj)(TILE(k, k + 1)), tau,
                              b, 1);
        if (!keep)
            for (int i = 0; i < b; ++i)
                for (int t = i + 1; t < b; ++t) *OSUF(oel)(TILE(k, k + 1), i, t) = 0;
        /* LQandmulQt2!: LQ2! = QR2! on adjoints, LQtapply2_par!, tile .= 0 */
        for (int64_t col = k + 2; col < nt; ++col) {
            OSUF(oracle_tsqrt_v)(OSUF(ov_adj)(TILE(k, k + 1)), OSUF(ov_adj)(TILE(k, col)), b, tau);
            KEEP_TAU(tp, k, col);
            OSUF(oracle_apply2_v)(OSUF(ov_adj)(TILE(k + 1, k + 1)), OSUF(ov_adj)(TILE(k + 1, col)),
                                  (nt - k - 1) * b, OSUF(ov_adj)(TILE(k, col)), tau, b, 1);
            if (!keep)
                for (int j = 0; j < b; ++j)
                    for (int t = 0; t < b; ++t) *OSUF(oel)(TILE(k, col), t, j) = 0;
        }
    }
#undef KEEP_TAU
#undef TILE
    free(tau);
}

void OSUF(oracle_blockbidiag)(OT *a, int64_t n, int64_t lda, int b) {
    OSUF(blockbidiag_impl)(a, n, lda, b, 0, NULL, NULL);
}

void OSUF(oracle_blockbidiag_keep)(OT *a, int64_t n, int64_t lda, int b, OT *tq, OT *tp) {
    OSUF(blockbidiag_impl)(a, n, lda, b, 1, tq, tp);
}

/*
 * Unblocked Householder QR of an m x p view with LAPACK-style reflectors
 * (beta = -sign(alpha) * norm, tau = (beta - alpha) / beta): the arithmetic of
 * Julia's qr! on the views that bulgechasing.jl:1-13 factors.  Only R is kept:
 * the reflector storage is overwritten with exact zeros (the triu! of QR_col!
 * and the triu/adjoint copy-back of QR_row!).  Reflectors are applied to the
 * remaining columns in parallel.
 */
void OSUF(oracle_house_qr_keep_r)(OSUF(oview) X, int64_t m, int64_t p) {
    int64_t kmax = m < p ? m : p;
    for (int64_t k = 0; k < kmax; ++k) {
        double s = 0;
        for (int64_t t = k + 1; t < m; ++t) {
            double x = (double)*OSUF(oel)(X, t, k);
            s += x * x;
        }
        if (s == 0.0) continue; /* H = I (LAPACK dlarfg with x == 0) */
        OT alpha = *OSUF(oel)(X, k, k);
        OT nrm = (OT)sqrt((double)alpha * (double)alpha + s);
        OT beta = alpha >= 0 ? -nrm : nrm;
        OT tauk = (beta - alpha) / beta;
        OT scal = (OT)1 / (alpha - beta);
        for (int64_t t = k + 1; t < m; ++t) *OSUF(oel)(X, t, k) *= scal;
        *OSUF(oel)(X, k, k) = beta;
        int64_t ncol = p - k - 1;
#pragma omp parallel for schedule(static) if (ncol * (m - k) >= 16384)
        for (int64_t j = k + 1; j < p; ++j) {
            OT w = *OSUF(oel)(X, k, j);
            for (int64_t t = k + 1; t < m; ++t) w += *OSUF(oel)(X, t, k) * *OSUF(oel)(X, t, j);
            w *= tauk;
            *OSUF(oel)(X, k, j) -= w;
            for (int64_t t = k + 1; t < m; ++t) *OSUF(oel)(X, t, j) -= w * *OSUF(oel)(X, t, k);
        }
        for (int64_t t = k + 1; t < m; ++t) *OSUF(oel)(X, t, k) = 0;
    }
}

/* QR_row! (bulgechasing.jl:1-7), 1-based inclusive indices as in the reference:
 * LQ of A[s:l, s+g:l], keep L. */
static void OSUF(o_qr_row)(OSUF(oview) A, int64_t s, int64_t l, int64_t g) {
    int64_t m = l - s + 1, p = l - (s + g) + 1;
    if (m <= 0 || p <= 0) return;
    OSUF(oview) X = OSUF(ov_sub)(A, s - 1, s + g - 1);
    OSUF(oracle_house_qr_keep_r)(OSUF(ov_adj)(X), p, m);
}

/* QR_col! (bulgechasing.jl:9-13): QR of A[s:l, s:l+g], keep R. */
static void OSUF(o_qr_col)(OSUF(oview) A, int64_t s, int64_t l, int64_t g) {
    int64_t m = l - s + 1, p = l + g - s + 1;
    if (m <= 0 || p <= 0) return;
    OSUF(oracle_house_qr_keep_r)(OSUF(ov_sub)(A, s - 1, s - 1), m, p);
}

/* block_bidiagonalize! (bulgechasing.jl:17-31), 1-based loop bounds kept. */
void OSUF(oracle_block_bidiagonalize)(OT *a, int64_t n, int64_t lda, int64_t bw, int64_t tbw) {
    OSUF(oview) A = OSUF(ov_cm)(a, lda);
    for (int64_t j = 1; j <= n - tbw; j += tbw) {
        int64_t l0 = j + bw + tbw - 1;
        OSUF(o_qr_row)(A, j, l0 < n ? l0 : n, tbw);
        for (int64_t i = j; i <= n; i += bw) {
            int64_t last = i + bw + tbw - 1;
            if (last > n) last = n;
            int64_t r = n - i - bw - tbw + 1;
            if (r < 0) r = 0;
            int64_t sc = bw + tbw - 1;
            if (r < sc) sc = r;
            OSUF(o_qr_col)(A, i + tbw, last, sc);
            if (i + tbw > n - bw) break;
            OSUF(o_qr_row)(A, i + tbw, last + sc, bw);
        }
    }
}

/* bidiagonalize (bulgechasing.jl:33-42): halve the band while it exceeds 16,
 * then chase the last band down to one superdiagonal. */
void OSUF(oracle_bidiagonalize)(OT *a, int64_t n, int64_t lda, int64_t bw) {
    while (bw > 16) {
        bw = (bw + 1) / 2; /* round(Int, bw/2) for the power-of-two bands used here */
        OSUF(oracle_block_bidiagonalize)(a, n, lda, 2 * bw, bw);
    }
    OSUF(oracle_block_bidiagonalize)(a, n, lda, bw, 1);
}

#undef OSUF
#undef OSUF1
#undef OSUF2
