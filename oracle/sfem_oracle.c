/*
 * CPU oracle for the smearFEM.jl hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A C restatement of the reference's assembly and solve, used (1) by the
 * tests as the checker at sizes the NumPy restatement is too slow for, and
 * (2) by bench.py as the timed CPU baseline ("port").  The GPU library never
 * links or calls it.
 *
 *   oc_assemble   src/fem.jl:135-256: element loop in ascending e, Gauss
 *                 points in the order of src/fem.jl:161-176, Jac = coords*dN,
 *                 w = wgp*|det Jac|, dNdX = dN*inv(Jac), Ke = ((B'D)B)w added
 *                 into the element's COO slots (index layout of :203 and
 *                 :242), then COO -> CSC with Julia's sparse(I,J,V)
 *                 semantics (:253): rows bucketed in input order, duplicates
 *                 folded left in input order, explicit zeros kept, row indices
 *                 sorted per column.
 *   oc_solve_pcg  examples/vector3D.jl:315-322 with the dense inverse of
 *                 K_free replaced by Jacobi-preconditioned CG on the free
 *                 DOFs (the dense inverse is O(n_f^3) and infeasible beyond a
 *                 few 10^4 DOFs).  q = q_d + C q_f.  oc_pcg_begin / _run /
 *                 _end split the same solve into resumable pieces.
 *
 * Element work runs in parallel over elements (OpenMP) when nthreads > 1;
 * each element owns its COO slots, so results do not depend on the thread
 * count.  The COO -> CSC conversion is serial like Julia's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int64_t m, n, nnz;
    int64_t *colptr, *rowval; /* 1-based, like SparseMatrixCSC */
    double *nzval;
    /* CSR copy of K (0-based) built lazily for the solver */
    int64_t *rp, *cj;
    double *rv;
} oc_csc;

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ---- src/fem.jl:21-31 and :149-177 ------------------------------------- */
static void gauss_points(int ndim, double pts[8][3], double w[8]) {
    double a = -1.0, b = 1.0;
    double x0 = -(b - a) / (2 * sqrt(3.0)) + (b + a) / 2;
    double x1 = (b - a) / (2 * sqrt(3.0)) + (b + a) / 2;
    double w0 = (b - a) / 2, w1 = (b - a) / 2;
    static const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    static const int oy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    static const int oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    int ng = ndim == 2 ? 4 : 8;
    for (int g = 0; g < ng; ++g) {
        pts[g][0] = ox[g] ? x1 : x0;
        pts[g][1] = oy[g] ? x1 : x0;
        pts[g][2] = oz[g] ? x1 : x0;
        double wx = ox[g] ? w1 : w0, wy = oy[g] ? w1 : w0, wz = oz[g] ? w1 : w0;
        w[g] = ndim == 2 ? wx * wy : wx * wy * wz;
    }
}

/* ---- src/fem.jl:48-111: reference gradients dN[a][k] ------------------- */
static void basis_grad(int ndim, int fclass, const double *p, double dN[9][3]) {
    double x = p[0], y = p[1], z = p[2];
    if (fclass == 1 && ndim == 3) {
        double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
        double sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
        double sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
        for (int a = 0; a < 8; ++a) {
            dN[a][0] = sx[a] * (1 + sy[a] * y) * (1 + sz[a] * z) / 8;
            dN[a][1] = sy[a] * (1 + sx[a] * x) * (1 + sz[a] * z) / 8;
            dN[a][2] = sz[a] * (1 + sx[a] * x) * (1 + sy[a] * y) / 8;
        }
    } else if (fclass == 1) {
        double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
        for (int a = 0; a < 4; ++a) {
            dN[a][0] = sx[a] * (1 + sy[a] * y) / 4;
            dN[a][1] = sy[a] * (1 + sx[a] * x) / 4;
        }
    } else { /* Q2, 9 nodes: corners, edge mids (bottom, right, top, left), centre */
        dN[0][0] = (1 - 2 * x) * (1 - y) * y / 4;   dN[0][1] = (1 - x) * x * (1 - 2 * y) / 4;
        dN[1][0] = -(1 + 2 * x) * (1 - y) * y / 4;  dN[1][1] = -x * (1 + x) * (1 - 2 * y) / 4;
        dN[2][0] = (1 + 2 * x) * y * (1 + y) / 4;   dN[2][1] = x * (1 + x) * (1 + 2 * y) / 4;
        dN[3][0] = -(1 - 2 * x) * y * (1 + y) / 4;  dN[3][1] = -(1 - x) * x * (1 + 2 * y) / 4;
        dN[4][0] = x * (1 - y) * y;                 dN[4][1] = -(1 - x) * (1 + x) * (1 - 2 * y) / 2;
        dN[5][0] = (1 + 2 * x) * (1 - y) * (1 + y) / 2; dN[5][1] = -x * (1 + x) * y;
        dN[6][0] = -x * y * (1 + y);                dN[6][1] = (1 - x) * (1 + x) * (1 + 2 * y) / 2;
        dN[7][0] = -(1 - 2 * x) * (1 - y) * (1 + y) / 2; dN[7][1] = (1 - x) * x * y;
        dN[8][0] = -2 * x * (1 - y) * (1 + y);      dN[8][1] = -(1 - x) * (1 + x) * 2 * y;
    }
}

/* D of src/fem.jl:217 (plane stress), :230 (3D); plane strain is an extension */
static void dmat(int ndim, int plane, double E, double nu, double D[6][6]) {
    memset(D, 0, sizeof(double) * 36);
    if (ndim == 2 && plane == 0) {
        D[0][0] = E / (1 - nu * nu); D[0][1] = nu * E / (1 - nu * nu);
        D[1][0] = nu * E / (1 - nu * nu); D[1][1] = E / (1 - nu * nu);
        D[2][2] = E / (2 * (1 + nu));
    } else if (ndim == 2) {
        double c = E / ((1 + nu) * (1 - 2 * nu));
        D[0][0] = (1 - nu) * c; D[0][1] = nu * c; D[1][0] = nu * c; D[1][1] = (1 - nu) * c;
        D[2][2] = (1 - 2 * nu) / 2 * c;
    } else {
        double c = E / ((1 + nu) * (1 - 2 * nu));
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) D[i][j] = (i == j ? 1 - nu : nu) * c;
        for (int i = 3; i < 6; ++i) D[i][i] = (1 - 2 * nu) / 2 * c;
    }
}

/* Julia sparse(I,J,V): see the file header. I, J 1-based. */
static oc_csc *coo_to_csc(int64_t L, const int64_t *I, const int64_t *J, const double *V) {
    oc_csc *K = (oc_csc *)calloc(1, sizeof(oc_csc));
    int64_t m = 0, n = 0;
    for (int64_t k = 0; k < L; ++k) {
        if (I[k] > m) m = I[k];
        if (J[k] > n) n = J[k];
    }
    K->m = m; K->n = n;
    int64_t *Rp = (int64_t *)calloc((size_t)m + 2, sizeof(int64_t));
    for (int64_t k = 0; k < L; ++k) Rp[I[k] + 1]++;
    for (int64_t i = 0; i < m; ++i) Rp[i + 2] += Rp[i + 1];
    /* Rp[i+1] = start of row i (0-based i), used as a cursor */
    int64_t *Rj = (int64_t *)malloc(sizeof(int64_t) * (size_t)(L ? L : 1));
    double *Rx = (double *)malloc(sizeof(double) * (size_t)(L ? L : 1));
    for (int64_t k = 0; k < L; ++k) {
        int64_t p = Rp[I[k]]++;
        Rj[p] = J[k] - 1;
        Rx[p] = V[k];
    }
    /* now Rp[i] = start of row i */
    int64_t *mark = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    for (int64_t j = 0; j < n; ++j) mark[j] = -1;
    int64_t *Rlen = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    int64_t write = 0;
    for (int64_t i = 0; i < m; ++i) {
        int64_t rs = Rp[i], re = Rp[i + 1], ws = write;
        for (int64_t r = rs; r < re; ++r) {
            int64_t j = Rj[r];
            if (mark[j] < ws) {
                mark[j] = write;
                Rj[write] = j;
                Rx[write] = Rx[r];
                ++write;
            } else {
                Rx[mark[j]] += Rx[r]; /* left fold in input order */
            }
        }
        Rlen[i] = write - ws;
    }
    int64_t nnz = write;
    K->nnz = nnz;
    K->colptr = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    K->rowval = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    K->nzval = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    int64_t *cnt = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t k = 0; k < nnz; ++k) cnt[Rj[k] + 1]++;
    for (int64_t j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
    int64_t pos = 0;
    for (int64_t i = 0; i < m; ++i) {
        for (int64_t r = pos; r < pos + Rlen[i]; ++r) {
            int64_t q = cnt[Rj[r]]++;
            K->rowval[q] = i + 1;
            K->nzval[q] = Rx[r];
        }
        pos += Rlen[i];
    }
    K->colptr[0] = 1;
    for (int64_t j = 0; j < n; ++j) K->colptr[j + 1] = cnt[j] + 1;
    free(Rp); free(Rj); free(Rx); free(mark); free(Rlen); free(cnt);
    return K;
}

void *oc_assemble(int ndim, int nen, int64_t nEl, int nDof, int fclass, int plane,
                  const double *NodeList, int64_t nN, const int64_t *IEN, int64_t ldIEN,
                  const int64_t *ID, const double *Ev, int64_t nE, const double *nuv,
                  int64_t nNu, int nthreads, double *t_elem, double *t_sparse) {
    (void)nN;
    if (ndim < 2 || ndim > 3) return NULL;
    if (nDof != 1 && nDof != ndim) return NULL;
    int ng = ndim == 2 ? 4 : 8;
    int nk = nDof * nen;
    int64_t per = (int64_t)nk * nk;
    int64_t L = nEl * per;
    int64_t *I = (int64_t *)calloc((size_t)(L ? L : 1), sizeof(int64_t));
    int64_t *J = (int64_t *)calloc((size_t)(L ? L : 1), sizeof(int64_t));
    double *V = (double *)calloc((size_t)(L ? L : 1), sizeof(double));
    double pts[8][3], wg[8];
    gauss_points(ndim, pts, wg);
    double t0 = now_s();
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static) if (nthreads > 1)
#endif
    for (int64_t e = 0; e < nEl; ++e) {
        double X[9][3];
        int64_t node[9];
        for (int a = 0; a < nen; ++a) {
            node[a] = IEN[e + (int64_t)a * ldIEN];
            for (int i = 0; i < ndim; ++i) X[a][i] = NodeList[(node[a] - 1) * ndim + i];
        }
        double E = Ev[nE > 1 ? e : 0], nu = nuv[nNu > 1 ? e : 0];
        double D[6][6];
        if (nDof > 1) dmat(ndim, plane, E, nu, D);
        int64_t base = e * per;
        for (int g = 0; g < ng; ++g) {
            double dN[9][3];
            basis_grad(ndim, fclass, pts[g], dN);
            double Jm[3][3] = {{0}};
            for (int i = 0; i < ndim; ++i)
                for (int k = 0; k < ndim; ++k) {
                    double s = 0;
                    for (int a = 0; a < nen; ++a) s += X[a][i] * dN[a][k];
                    Jm[i][k] = s;
                }
            double det, inv[3][3];
            if (ndim == 2) {
                det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
                inv[0][0] = Jm[1][1] / det; inv[0][1] = -Jm[0][1] / det;
                inv[1][0] = -Jm[1][0] / det; inv[1][1] = Jm[0][0] / det;
            } else {
                double c00 = Jm[1][1] * Jm[2][2] - Jm[1][2] * Jm[2][1];
                double c01 = Jm[1][2] * Jm[2][0] - Jm[1][0] * Jm[2][2];
                double c02 = Jm[1][0] * Jm[2][1] - Jm[1][1] * Jm[2][0];
                det = Jm[0][0] * c00 + Jm[0][1] * c01 + Jm[0][2] * c02;
                inv[0][0] = c00 / det;
                inv[0][1] = (Jm[0][2] * Jm[2][1] - Jm[0][1] * Jm[2][2]) / det;
                inv[0][2] = (Jm[0][1] * Jm[1][2] - Jm[0][2] * Jm[1][1]) / det;
                inv[1][0] = c01 / det;
                inv[1][1] = (Jm[0][0] * Jm[2][2] - Jm[0][2] * Jm[2][0]) / det;
                inv[1][2] = (Jm[0][2] * Jm[1][0] - Jm[0][0] * Jm[1][2]) / det;
                inv[2][0] = c02 / det;
                inv[2][1] = (Jm[0][1] * Jm[2][0] - Jm[0][0] * Jm[2][1]) / det;
                inv[2][2] = (Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0]) / det;
            }
            double w = wg[g] * fabs(det);
            double G[9][3];
            for (int a = 0; a < nen; ++a)
                for (int k = 0; k < ndim; ++k) {
                    double s = 0;
                    for (int j = 0; j < ndim; ++j) s += dN[a][j] * inv[j][k];
                    G[a][k] = s;
                }
            if (nDof == 1) {
                for (int i = 0; i < nen; ++i)
                    for (int j = 0; j < nen; ++j) {
                        int64_t inz = base + (int64_t)nen * i + j;
                        double s = 0;
                        for (int k = 0; k < ndim; ++k) s += G[i][k] * G[j][k];
                        I[inz] = node[i];
                        J[inz] = node[j];
                        V[inz] += w * s;
                    }
            } else {
                int ns = ndim == 2 ? 3 : 6;
                double B[6][27];
                memset(B, 0, sizeof(B));
                for (int a = 0; a < nen; ++a) {
                    if (ndim == 2) {
                        B[0][2 * a] = G[a][0]; B[1][2 * a + 1] = G[a][1];
                        B[2][2 * a] = G[a][1]; B[2][2 * a + 1] = G[a][0];
                    } else {
                        B[0][3 * a] = G[a][0]; B[1][3 * a + 1] = G[a][1]; B[2][3 * a + 2] = G[a][2];
                        B[3][3 * a + 1] = G[a][2]; B[3][3 * a + 2] = G[a][1];
                        B[4][3 * a] = G[a][2]; B[4][3 * a + 2] = G[a][0];
                        B[5][3 * a] = G[a][1]; B[5][3 * a + 1] = G[a][0];
                    }
                }
                double BtD[27][6];
                for (int i = 0; i < nk; ++i)
                    for (int s = 0; s < ns; ++s) {
                        double acc = 0;
                        for (int r = 0; r < ns; ++r) acc += B[r][i] * D[r][s];
                        BtD[i][s] = acc;
                    }
                for (int iN = 0; iN < nen; ++iN)
                    for (int jN = 0; jN < nen; ++jN)
                        for (int iD = 0; iD < nDof; ++iD)
                            for (int jD = 0; jD < nDof; ++jD) {
                                int i = iN * nDof + iD, j = jN * nDof + jD;
                                double acc = 0;
                                for (int s = 0; s < ns; ++s) acc += BtD[i][s] * B[s][j];
                                int64_t inz = base + (int64_t)iN * nDof * nk + (int64_t)jN * nDof * nDof +
                                              iD * nDof + jD;
                                I[inz] = ID[(node[iN] - 1) + (int64_t)iD * nN];
                                J[inz] = ID[(node[jN] - 1) + (int64_t)jD * nN];
                                V[inz] += acc * w;
                            }
            }
        }
    }
    double t1 = now_s();
    oc_csc *K = coo_to_csc(L, I, J, V);
    double t2 = now_s();
    free(I); free(J); free(V);
    if (t_elem) *t_elem = t1 - t0;
    if (t_sparse) *t_sparse = t2 - t1;
    return K;
}

void oc_csc_info(void *h, int64_t *m, int64_t *n, int64_t *nnz) {
    oc_csc *K = (oc_csc *)h;
    *m = K->m; *n = K->n; *nnz = K->nnz;
}

void oc_csc_copy(void *h, int64_t *colptr, int64_t *rowval, double *nzval) {
    oc_csc *K = (oc_csc *)h;
    if (colptr) memcpy(colptr, K->colptr, sizeof(int64_t) * (size_t)(K->n + 1));
    if (rowval) memcpy(rowval, K->rowval, sizeof(int64_t) * (size_t)K->nnz);
    if (nzval) memcpy(nzval, K->nzval, sizeof(double) * (size_t)K->nnz);
}

/* Wrap caller-provided CSC arrays (1-based) without assembling. */
void *oc_csc_wrap(int64_t n, int64_t nnz, const int64_t *colptr, const int64_t *rowval,
                  const double *nzval) {
    oc_csc *K = (oc_csc *)calloc(1, sizeof(oc_csc));
    K->m = K->n = n; K->nnz = nnz;
    K->colptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    K->rowval = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    K->nzval = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    memcpy(K->colptr, colptr, sizeof(int64_t) * (size_t)(n + 1));
    memcpy(K->rowval, rowval, sizeof(int64_t) * (size_t)nnz);
    memcpy(K->nzval, nzval, sizeof(double) * (size_t)nnz);
    return K;
}

void oc_free(void *h) {
    oc_csc *K = (oc_csc *)h;
    if (!K) return;
    free(K->colptr); free(K->rowval); free(K->nzval);
    free(K->rp); free(K->cj); free(K->rv);
    free(K);
}

/* CSR of K (transpose of the stored CSC), 0-based.  K's pattern is
 * symmetric (every element writes the full node-pair block), so row i of the
 * CSR has the pattern of column i, and entry (i, j) of column j goes to the
 * position of j in column i's sorted row list: each column is transposed
 * independently (parallel, no conflicts).  A non-symmetric pattern takes the
 * serial counting transposition. */
static int64_t find_sorted(const int64_t *a, int64_t lo, int64_t hi, int64_t v) {
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

static void build_csr(oc_csc *K) {
    if (K->rp) return;
    int64_t n = K->n, m = K->m, nnz = K->nnz;
    K->rp = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    K->cj = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz ? nnz : 1));
    K->rv = (double *)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
    int sym = (m == n);
    if (sym) {
        int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4096) reduction(| : bad)
#endif
        for (int64_t j = 0; j < n; ++j) {
            for (int64_t k = K->colptr[j] - 1; k < K->colptr[j + 1] - 1; ++k) {
                int64_t i = K->rowval[k] - 1; /* entry (i, j) */
                int64_t a = K->colptr[i] - 1, b = K->colptr[i + 1] - 1;
                int64_t q = find_sorted(K->rowval, a, b, j + 1);
                if (q >= b || K->rowval[q] != j + 1) {
                    bad = 1;
                    continue;
                }
                K->cj[q] = j;
                K->rv[q] = K->nzval[k];
            }
        }
        if (!bad) {
            for (int64_t i = 0; i <= m; ++i) K->rp[i] = K->colptr[i] - 1;
            return;
        }
        memset(K->rp, 0, sizeof(int64_t) * (size_t)(m + 1));
    }
    for (int64_t k = 0; k < nnz; ++k) K->rp[K->rowval[k]]++;
    for (int64_t i = 0; i < m; ++i) K->rp[i + 1] += K->rp[i];
    int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m + 1));
    memcpy(cur, K->rp, sizeof(int64_t) * (size_t)(m + 1));
    for (int64_t j = 0; j < n; ++j)
        for (int64_t k = K->colptr[j] - 1; k < K->colptr[j + 1] - 1; ++k) {
            int64_t q = cur[K->rowval[k] - 1]++;
            K->cj[q] = j;
            K->rv[q] = K->nzval[k];
        }
    free(cur);
}

/* y = mask .* (K x), K in CSR */
static void spmv(const oc_csc *K, const double *x, double *y, const unsigned char *fixed, int nth) {
    (void)nth;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (nth > 1)
#endif
    for (int64_t i = 0; i < K->m; ++i) {
        double s = 0;
        for (int64_t k = K->rp[i]; k < K->rp[i + 1]; ++k) s += K->rv[k] * x[K->cj[k]];
        y[i] = (fixed && fixed[i]) ? 0.0 : s;
    }
}

static double dot(int64_t n, const double *a, const double *b, int nth) {
    (void)nth;
    double s = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) schedule(static) if (nth > 1)
#endif
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/*
 * Dirichlet elimination + Jacobi-PCG (examples/vector3D.jl:315-322 with the
 * dense inverse replaced), as a resumable solve:
 *   oc_pcg_begin  lift (r = C'(f - K q_d)), Jacobi diagonal, z = M^-1 r, p = z
 *   oc_pcg_run    up to max_iters more CG iterations, or until the relative
 *                 residual is at or below rtol
 *   oc_pcg_end    q = q_d + C q_f, statistics, frees the state
 * Splitting a solve into several oc_pcg_run calls performs exactly the
 * iterations of one call.  fixed: 1-based DOF ids.
 */
typedef struct {
    oc_csc *K;
    int64_t n;
    int nth, it, status; /* status: 0 converged, 1 running / maxit, 2 zero diagonal */
    unsigned char *fx;
    double *ud, *r, *z, *p, *q, *x, *dinv;
    double bb, rr, rz, t0;
} oc_pcg;

void *oc_pcg_begin(void *h, const int64_t *fixed, int64_t nfix, const double *vals,
                   const double *f, int nthreads) {
    oc_pcg *S = (oc_pcg *)calloc(1, sizeof(oc_pcg));
    oc_csc *K = (oc_csc *)h;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    S->t0 = now_s();
    S->K = K;
    S->nth = nthreads;
    build_csr(K);
    int64_t n = S->n = K->n;
    S->fx = (unsigned char *)calloc((size_t)n, 1);
    S->ud = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t k = 0; k < nfix; ++k) {
        S->fx[fixed[k] - 1] = 1;
        S->ud[fixed[k] - 1] = vals[k];
    }
    S->r = (double *)malloc(sizeof(double) * (size_t)n);
    S->z = (double *)malloc(sizeof(double) * (size_t)n);
    S->p = (double *)malloc(sizeof(double) * (size_t)n);
    S->q = (double *)malloc(sizeof(double) * (size_t)n);
    S->x = (double *)calloc((size_t)n, sizeof(double));
    S->dinv = (double *)calloc((size_t)n, sizeof(double));
    unsigned char *fx = S->fx;
    double *dinv = S->dinv;
    int status = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : status) if (nthreads > 1)
#endif
    for (int64_t i = 0; i < n; ++i) {
        if (fx[i]) continue;
        double d = 0;
        for (int64_t k = K->rp[i]; k < K->rp[i + 1]; ++k)
            if (K->cj[k] == i) d += K->rv[k];
        if (d == 0) status |= 2;
        dinv[i] = d != 0 ? 1.0 / d : 0.0;
    }
    spmv(K, S->ud, S->q, fx, nthreads);
    for (int64_t i = 0; i < n; ++i) S->r[i] = fx[i] ? 0.0 : (f ? f[i] : 0.0) - S->q[i];
    S->bb = S->rr = dot(n, S->r, S->r, nthreads);
    if (status == 0 && S->bb > 0) {
        for (int64_t i = 0; i < n; ++i) { S->z[i] = dinv[i] * S->r[i]; S->p[i] = S->z[i]; }
        S->rz = dot(n, S->r, S->z, nthreads);
        status = 1;
    }
    S->status = status;
    return S;
}

/* Returns the status (0 once converged).  mark_rtol > 0: the first
 * iteration at which the relative residual is at or below mark_rtol, and
 * the seconds since oc_pcg_begin started, go to *mark_iters / *mark_s (left
 * alone while it is not reached, so *mark_iters starts at -1). */
int oc_pcg_run(void *state, int max_iters, double rtol, double mark_rtol, int *mark_iters,
               double *mark_s) {
    oc_pcg *S = (oc_pcg *)state;
    const int64_t n = S->n;
    const int nthreads = S->nth;
    double *x = S->x, *r = S->r, *z = S->z, *p = S->p, *q = S->q, *dinv = S->dinv;
    if (S->status != 1) return S->status;
    if (S->rr <= rtol * rtol * S->bb) { S->status = 0; return 0; }
    for (int k = 0; k < max_iters; ++k) {
        spmv(S->K, p, q, S->fx, nthreads);
        double alpha = S->rz / dot(n, p, q, nthreads);
        double rzn = 0, rrn = 0;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : rzn, rrn) schedule(static) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
            rzn += r[i] * z[i];
            rrn += r[i] * r[i];
        }
        ++S->it;
        S->rr = rrn;
        if (mark_rtol > 0 && mark_iters && *mark_iters < 0 && S->rr <= mark_rtol * mark_rtol * S->bb) {
            *mark_iters = S->it;
            if (mark_s) *mark_s = now_s() - S->t0;
        }
        if (S->rr <= rtol * rtol * S->bb) { S->status = 0; return 0; }
        double beta = rzn / S->rz;
        S->rz = rzn;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    return S->status;
}

int oc_pcg_end(void *state, double *u, int *iters, double *relres, double *t_solve) {
    oc_pcg *S = (oc_pcg *)state;
    int status = S->status;
    for (int64_t i = 0; i < S->n; ++i) u[i] = S->ud[i] + S->x[i];
    if (iters) *iters = S->it;
    if (relres) *relres = S->bb > 0 ? sqrt(S->rr / S->bb) : 0.0;
    if (t_solve) *t_solve = now_s() - S->t0;
    free(S->fx); free(S->ud); free(S->r); free(S->z); free(S->p); free(S->q); free(S->x);
    free(S->dinv);
    free(S);
    return status;
}

/* The whole solve in one call.  Returns 0 on success, 1 if maxit was reached,
 * 2 on a zero diagonal at a free DOF; mark_rtol as in oc_pcg_run
 * (*mark_iters = -1 if it was never reached). */
int oc_solve_pcg_mark(void *h, const int64_t *fixed, int64_t nfix, const double *vals,
                      const double *f, double rtol, int maxit, int nthreads, double *u,
                      int *iters, double *relres, double *t_solve, double mark_rtol,
                      int *mark_iters, double *mark_s) {
    if (mark_iters) *mark_iters = -1;
    if (mark_s) *mark_s = 0.0;
    void *S = oc_pcg_begin(h, fixed, nfix, vals, f, nthreads);
    oc_pcg *P = (oc_pcg *)S;
    if (P->status == 1 && mark_rtol > 0 && P->rr <= mark_rtol * mark_rtol * P->bb && mark_iters) {
        *mark_iters = 0;
        if (mark_s) *mark_s = now_s() - P->t0;
    }
    oc_pcg_run(S, maxit, rtol, mark_rtol, mark_iters, mark_s);
    return oc_pcg_end(S, u, iters, relres, t_solve);
}

int oc_solve_pcg(void *h, const int64_t *fixed, int64_t nfix, const double *vals,
                 const double *f, double rtol, int maxit, int nthreads, double *u,
                 int *iters, double *relres, double *t_solve) {
    return oc_solve_pcg_mark(h, fixed, nfix, vals, f, rtol, maxit, nthreads, u, iters, relres,
                             t_solve, 0.0, NULL, NULL);
}

int oc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
