/*
 * oracle.c -- CPU restatement of the schwarz-gmres solve path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See oracle.h for the contract.
 * Each function cites the reference file:line it restates; operation order
 * follows the reference so that results are bit-identical to the reference
 * build on the same host (compiled with -ffp-contract=off).
 *
 * Parallelism mirrors the reference: SpMV, BLAS-1 and the Arnoldi loop are
 * serial (src/core/sparse_matrix.h:30-37, src/core/vector.h, src/core/
 * gmres.cpp); the Schwarz applies run the subdomain loop under OpenMP
 * (src/precond/ras.h:48, src/precond/asm.h:38).
 */
#include "oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_free(void* p) { free(p); }

/* ---------------------------------------------------------------- BLAS-1 */
/* src/core/vector.h:11-16 */
static double o_dot(const double* a, const double* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
/* src/core/vector.h:23-25 */
static double o_norm2(const double* a, int n) { return sqrt(o_dot(a, a, n)); }
/* src/core/vector.h:31-34 */
static void o_axpy(double alpha, const double* x, double* y, int n) {
    for (int i = 0; i < n; ++i) y[i] += alpha * x[i];
}

/* ---------------------------------------------------------------- CSR */
/* src/core/sparse_matrix.h:30-37: serial row loop, sum from 0.0 in entry order */
void orc_spmv(int n, const int* rp, const int* ci, const double* v,
              const double* x, double* y) {
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int e = rp[i]; e < rp[i + 1]; ++e) s += v[e] * x[ci[e]];
        y[i] = s;
    }
}

/* src/core/sparse_matrix.h:53-83: inverse map over max(nrows,ncols); rows in
 * idx order, entries kept in their original column order. */
int orc_extract(int nrows, int ncols, const int* rp, const int* ci, const double* v,
                const int* idx, int nidx, int* rp_out, int* ci_out, double* v_out) {
    int span = nrows > ncols ? nrows : ncols;
    int* inv = (int*)malloc(sizeof(int) * (size_t)(span > 0 ? span : 1));
    for (int i = 0; i < span; ++i) inv[i] = -1;
    for (int i = 0; i < nidx; ++i) inv[idx[i]] = i;
    int nz = 0;
    for (int li = 0; li < nidx; ++li) {
        int gi = idx[li];
        if (rp_out) rp_out[li] = nz;
        for (int e = rp[gi]; e < rp[gi + 1]; ++e) {
            int lj = inv[ci[e]];
            if (lj >= 0) {
                if (ci_out) { ci_out[nz] = lj; v_out[nz] = v[e]; }
                ++nz;
            }
        }
    }
    if (rp_out) rp_out[nidx] = nz;
    free(inv);
    return nz;
}

/* ---------------------------------------------------------------- ILU(0) */
/* src/precond/ilu0.h:13-54.  IKJ elimination on the CSR pattern; a pivot that
 * is absent or below 1e-30 in magnitude skips the row update; the matching
 * column in row i is found by linear search (first match). */
void orc_ilu0_factor(int n, const int* rp, const int* ci, const double* v,
                     double* lu, int* diag) {
    memcpy(lu, v, sizeof(double) * (size_t)rp[n]);
    for (int i = 0; i < n; ++i) {
        diag[i] = -1;
        for (int e = rp[i]; e < rp[i + 1]; ++e)
            if (ci[e] == i) { diag[i] = e; break; }
    }
    for (int i = 1; i < n; ++i) {
        for (int jp = rp[i]; jp < rp[i + 1]; ++jp) {
            int k = ci[jp];
            if (k >= i) break;
            int dk = diag[k];
            if (dk < 0 || fabs(lu[dk]) < 1e-30) continue;
            double a_ik = lu[jp] / lu[dk];
            lu[jp] = a_ik;
            for (int kp = dk + 1; kp < rp[k + 1]; ++kp) {
                int col = ci[kp];
                for (int ip = rp[i]; ip < rp[i + 1]; ++ip) {
                    if (ci[ip] == col) { lu[ip] -= a_ik * lu[kp]; break; }
                }
            }
        }
    }
}

/* src/precond/ilu0.h:57-79: unit-L forward sweep stopping at the first
 * column >= i, backward sweep from diag+1, divide by the diagonal. */
void orc_ilu0_solve(int n, const int* rp, const int* ci, const double* lu,
                    const int* diag, const double* x, double* y) {
    double* t = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    memcpy(t, x, sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        for (int jp = rp[i]; jp < rp[i + 1]; ++jp) {
            int col = ci[jp];
            if (col >= i) break;
            t[i] -= lu[jp] * t[col];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        for (int jp = diag[i] + 1; jp < rp[i + 1]; ++jp) t[i] -= lu[jp] * t[ci[jp]];
        t[i] /= lu[diag[i]];
    }
    memcpy(y, t, sizeof(double) * (size_t)n);
    free(t);
}

/* Dependency levels of the two sweeps above (row order is preserved). */
int orc_levels_lower(int n, const int* rp, const int* ci, int* level) {
    int nlev = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int e = rp[i]; e < rp[i + 1]; ++e) {
            int c = ci[e];
            if (c >= i) break;
            if (level[c] + 1 > l) l = level[c] + 1;
        }
        level[i] = l;
        if (l + 1 > nlev) nlev = l + 1;
    }
    return nlev;
}

int orc_levels_upper(int n, const int* rp, const int* ci, const int* diag, int* level) {
    int nlev = 0;
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int e = diag[i] + 1; e < rp[i + 1]; ++e) {
            int c = ci[e];
            if (level[c] + 1 > l) l = level[c] + 1;
        }
        level[i] = l;
        if (l + 1 > nlev) nlev = l + 1;
    }
    return nlev;
}

/* ---------------------------------------------------------------- decomposition */
/* src/decomp/domain_decomp.h:61-93.  owned_dofs[s] ascending; the overlap is
 * grown `overlap` times by every column of every row already in the set; the
 * final set is sorted.  The set after k layers is the set of vertices within
 * k hops of the owned set, so growing from the newest layer only gives the
 * same set.  The owned-local map is src/precond/ras.h:34-41. */
int orc_decompose(int n, const int* rp, const int* ci, const int* part, int nparts,
                  int overlap, int** owned_ptr_o, int** owned_o, int** sub_ptr_o,
                  int** sub_o, int** ownloc_ptr_o, int** ownloc_o) {
    if (nparts <= 0) return 1;
    for (int i = 0; i < n; ++i)
        if (part[i] < 0 || part[i] >= nparts) return 2;
    int* owned_ptr = (int*)calloc((size_t)nparts + 1, sizeof(int));
    for (int i = 0; i < n; ++i) owned_ptr[part[i] + 1]++;
    for (int s = 0; s < nparts; ++s) owned_ptr[s + 1] += owned_ptr[s];
    int* owned = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* fill = (int*)malloc(sizeof(int) * (size_t)nparts);
    memcpy(fill, owned_ptr, sizeof(int) * (size_t)nparts);
    for (int i = 0; i < n; ++i) owned[fill[part[i]]++] = i;
    free(fill);

    /* per-subdomain sets, built one after another */
    int cap = n > 16 ? n : 16;
    int total = 0, tcap = n + 16;
    int* sub = (int*)malloc(sizeof(int) * (size_t)tcap);
    int* sub_ptr = (int*)calloc((size_t)nparts + 1, sizeof(int));
    int* ownloc = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int* ownloc_ptr = (int*)calloc((size_t)nparts + 1, sizeof(int));
    unsigned char* mark = (unsigned char*)calloc((size_t)(n > 0 ? n : 1), 1);
    int* set = (int*)malloc(sizeof(int) * (size_t)cap);
    int nol = 0;
    for (int s = 0; s < nparts; ++s) {
        int ns = 0;
        for (int k = owned_ptr[s]; k < owned_ptr[s + 1]; ++k) {
            set[ns++] = owned[k];
            mark[owned[k]] = 1;
        }
        int lo = 0;
        for (int layer = 0; layer < overlap; ++layer) {
            int hi = ns;
            for (int q = lo; q < hi; ++q) {
                int r = set[q];
                for (int e = rp[r]; e < rp[r + 1]; ++e) {
                    int c = ci[e];
                    if (!mark[c]) { mark[c] = 1; set[ns++] = c; }
                }
            }
            lo = hi;
        }
        /* sorted: collect marks in index order over the touched entries */
        /* counting by a scan of the set then sort */
        {
            /* insertion into ascending order via marks is O(n); use qsort-free
             * two-pass: sort the small list with a radix-free approach */
            int* tmp = set;
            /* simple in-place sort (shell sort is fine for the oracle) */
            for (int gap = ns / 2; gap > 0; gap /= 2)
                for (int a = gap; a < ns; ++a) {
                    int val = tmp[a], b = a;
                    while (b >= gap && tmp[b - gap] > val) { tmp[b] = tmp[b - gap]; b -= gap; }
                    tmp[b] = val;
                }
        }
        if (total + ns > tcap) {
            while (total + ns > tcap) tcap *= 2;
            sub = (int*)realloc(sub, sizeof(int) * (size_t)tcap);
        }
        for (int q = 0; q < ns; ++q) {
            sub[total + q] = set[q];
            mark[set[q]] = 0;
        }
        /* owned-local indices: positions of owned dofs in the sorted set */
        for (int q = 0; q < ns; ++q)
            if (part[set[q]] == s) ownloc[nol++] = q;
        total += ns;
        sub_ptr[s + 1] = total;
        ownloc_ptr[s + 1] = nol;
    }
    free(mark);
    free(set);
    *owned_ptr_o = owned_ptr;
    *owned_o = owned;
    *sub_ptr_o = sub_ptr;
    *sub_o = sub;
    *ownloc_ptr_o = ownloc_ptr;
    *ownloc_o = ownloc;
    return 0;
}

/* ---------------------------------------------------------------- preconditioners */
typedef struct {
    int n, nnz;
    int* rp;
    int* ci;
    double* lu;
    int* diag;
} o_ilu;

struct orc_pc {
    int kind;
    int n;
    /* jacobi */
    double* inv_diag;
    /* single ILU0 */
    o_ilu ilu;
    /* schwarz */
    int nparts, overlap;
    int *owned_ptr, *owned, *sub_ptr, *sub, *ownloc_ptr, *ownloc;
    o_ilu* loc;
    /* coarse (two-level) */
    int nc;
    double* scale; /* 1/sqrt(|owned_s|) */
    double* a0;    /* nc*nc row-major, as built */
    double* lu0;   /* factored */
    int* piv;
};

static void o_ilu_setup(o_ilu* f, int n, const int* rp, const int* ci, const double* v) {
    f->n = n;
    f->nnz = rp[n];
    f->rp = (int*)malloc(sizeof(int) * (size_t)(n + 1));
    memcpy(f->rp, rp, sizeof(int) * (size_t)(n + 1));
    f->ci = (int*)malloc(sizeof(int) * (size_t)(f->nnz > 0 ? f->nnz : 1));
    memcpy(f->ci, ci, sizeof(int) * (size_t)f->nnz);
    f->lu = (double*)malloc(sizeof(double) * (size_t)(f->nnz > 0 ? f->nnz : 1));
    f->diag = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    orc_ilu0_factor(n, rp, ci, v, f->lu, f->diag);
}

static void o_ilu_free(o_ilu* f) {
    free(f->rp); free(f->ci); free(f->lu); free(f->diag);
}

/* src/precond/coarse_space.h:26-60 restated without the dense P x n R0.
 * R0[s][k] = c_s on owned dofs of s, zero elsewhere, so in the reference
 *   A_phi[j][k] = sum over entries of row k (entry order) of A_kl * R0[j][l]
 *   A0[i][j]    = sum over k ascending of R0[i][k] * A_phi[j][k]
 * and every term with a zero factor adds an exact zero.  Keeping only the
 * nonzero terms in the same order gives the same bits. */
static void o_build_coarse(orc_pc* pc, const int* rp, const int* ci, const double* v,
                           const int* part) {
    int nc = pc->nparts, n = pc->n;
    pc->nc = nc;
    pc->scale = (double*)malloc(sizeof(double) * (size_t)nc);
    for (int s = 0; s < nc; ++s)
        pc->scale[s] = 1.0 / sqrt((double)(pc->owned_ptr[s + 1] - pc->owned_ptr[s]));
    pc->a0 = (double*)calloc((size_t)nc * (size_t)nc, sizeof(double));
    /* per row k: partial sums keyed by part, in entry order */
    int* seen = (int*)malloc(sizeof(int) * (size_t)nc);
    double* acc = (double*)malloc(sizeof(double) * (size_t)nc);
    int* list = (int*)malloc(sizeof(int) * (size_t)nc);
    for (int s = 0; s < nc; ++s) seen[s] = -1;
    for (int i = 0; i < nc; ++i) {
        double ci_s = pc->scale[i];
        for (int q = pc->owned_ptr[i]; q < pc->owned_ptr[i + 1]; ++q) {
            int k = pc->owned[q];
            int nl = 0;
            for (int e = rp[k]; e < rp[k + 1]; ++e) {
                int j = part[ci[e]];
                if (seen[j] != k) { seen[j] = k; acc[j] = 0.0; list[nl++] = j; }
                acc[j] += v[e] * pc->scale[j];
            }
            for (int t = 0; t < nl; ++t) {
                int j = list[t];
                pc->a0[(size_t)i * nc + j] += ci_s * acc[j];
            }
        }
    }
    (void)n;
    free(seen); free(acc); free(list);
}

/* src/precond/coarse_solve.h:15-47: dense row-major LU, partial pivoting on
 * the first strictly larger magnitude, full row swaps. */
static int o_coarse_factor(orc_pc* pc) {
    int n = pc->nc;
    pc->lu0 = (double*)malloc(sizeof(double) * (size_t)n * (size_t)n);
    memcpy(pc->lu0, pc->a0, sizeof(double) * (size_t)n * (size_t)n);
    pc->piv = (int*)malloc(sizeof(int) * (size_t)n);
    double* L = pc->lu0;
    for (int k = 0; k < n; ++k) {
        int mr = k;
        double mv = fabs(L[(size_t)k * n + k]);
        for (int i = k + 1; i < n; ++i) {
            double a = fabs(L[(size_t)i * n + k]);
            if (a > mv) { mv = a; mr = i; }
        }
        pc->piv[k] = mr;
        if (mv < 1e-30) return 1;
        if (mr != k)
            for (int j = 0; j < n; ++j) {
                double t = L[(size_t)k * n + j];
                L[(size_t)k * n + j] = L[(size_t)mr * n + j];
                L[(size_t)mr * n + j] = t;
            }
        for (int i = k + 1; i < n; ++i) {
            L[(size_t)i * n + k] /= L[(size_t)k * n + k];
            for (int j = k + 1; j < n; ++j)
                L[(size_t)i * n + j] -= L[(size_t)i * n + k] * L[(size_t)k * n + j];
        }
    }
    return 0;
}

/* src/precond/coarse_solve.h:50-67 */
static void o_coarse_solve(const orc_pc* pc, const double* b, double* x) {
    int n = pc->nc;
    const double* L = pc->lu0;
    memcpy(x, b, sizeof(double) * (size_t)n);
    for (int k = 0; k < n; ++k) {
        if (pc->piv[k] != k) { double t = x[k]; x[k] = x[pc->piv[k]]; x[pc->piv[k]] = t; }
        for (int i = k + 1; i < n; ++i) x[i] -= L[(size_t)i * n + k] * x[k];
    }
    for (int k = n - 1; k >= 0; --k) {
        for (int j = k + 1; j < n; ++j) x[k] -= L[(size_t)k * n + j] * x[j];
        x[k] /= L[(size_t)k * n + k];
    }
}

orc_pc* orc_pc_create(int kind, int n, const int* rp, const int* ci, const double* v,
                      int nparts, int overlap, const int* part, int* err) {
    orc_pc* pc = (orc_pc*)calloc(1, sizeof(orc_pc));
    pc->kind = kind;
    pc->n = n;
    *err = 0;
    if (kind == ORC_PC_NONE) return pc;
    if (kind == ORC_PC_JACOBI) {
        /* src/precond/jacobi.h:12-17 and sparse_matrix.h:45-51 */
        pc->inv_diag = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        for (int i = 0; i < n; ++i) {
            double d = 0.0;
            for (int e = rp[i]; e < rp[i + 1]; ++e)
                if (ci[e] == i) { d = v[e]; break; }
            pc->inv_diag[i] = (fabs(d) > 1e-15) ? 1.0 / d : 1.0;
        }
        return pc;
    }
    if (kind == ORC_PC_ILU0) {
        o_ilu_setup(&pc->ilu, n, rp, ci, v);
        return pc;
    }
    /* Schwarz: src/precond/ras.h:21-43, asm.h:20-32 */
    pc->nparts = nparts;
    pc->overlap = overlap;
    if (orc_decompose(n, rp, ci, part, nparts, overlap, &pc->owned_ptr, &pc->owned,
                      &pc->sub_ptr, &pc->sub, &pc->ownloc_ptr, &pc->ownloc)) {
        *err = 2;
        return pc;
    }
    pc->loc = (o_ilu*)calloc((size_t)nparts, sizeof(o_ilu));
#pragma omp parallel for schedule(dynamic)
    for (int s = 0; s < nparts; ++s) {
        const int* idx = pc->sub + pc->sub_ptr[s];
        int ns = pc->sub_ptr[s + 1] - pc->sub_ptr[s];
        int nz = orc_extract(n, n, rp, ci, v, idx, ns, NULL, NULL, NULL);
        int* lrp = (int*)malloc(sizeof(int) * (size_t)(ns + 1));
        int* lci = (int*)malloc(sizeof(int) * (size_t)(nz > 0 ? nz : 1));
        double* lv = (double*)malloc(sizeof(double) * (size_t)(nz > 0 ? nz : 1));
        orc_extract(n, n, rp, ci, v, idx, ns, lrp, lci, lv);
        o_ilu_setup(&pc->loc[s], ns, lrp, lci, lv);
        free(lrp); free(lci); free(lv);
    }
    if (kind == ORC_PC_TWOLEVEL_ASM || kind == ORC_PC_TWOLEVEL_RAS) {
        /* src/precond/two_level_schwarz.h:29-48 */
        o_build_coarse(pc, rp, ci, v, part);
        if (o_coarse_factor(pc)) *err = 3;
    }
    return pc;
}

/* one subdomain solve: gather, ILU sweep (src/precond/ras.h:50-61) */
static void o_local_solve(const orc_pc* pc, int s, const double* x, double* z) {
    const int* dofs = pc->sub + pc->sub_ptr[s];
    int ns = pc->sub_ptr[s + 1] - pc->sub_ptr[s];
    double* r = (double*)malloc(sizeof(double) * (size_t)(ns > 0 ? ns : 1));
    for (int i = 0; i < ns; ++i) r[i] = x[dofs[i]];
    const o_ilu* f = &pc->loc[s];
    orc_ilu0_solve(ns, f->rp, f->ci, f->lu, f->diag, r, z);
    free(r);
}

static void o_fine_apply(const orc_pc* pc, const double* x, double* y, int n) {
    int restricted = (pc->kind == ORC_PC_RAS || pc->kind == ORC_PC_TWOLEVEL_RAS);
    for (int i = 0; i < n; ++i) y[i] = 0.0;
    if (restricted) {
        /* src/precond/ras.h:45-70: owned sets are disjoint, no lock */
#pragma omp parallel for schedule(dynamic)
        for (int s = 0; s < pc->nparts; ++s) {
            int ns = pc->sub_ptr[s + 1] - pc->sub_ptr[s];
            double* z = (double*)malloc(sizeof(double) * (size_t)(ns > 0 ? ns : 1));
            o_local_solve(pc, s, x, z);
            const int* dofs = pc->sub + pc->sub_ptr[s];
            for (int q = pc->ownloc_ptr[s]; q < pc->ownloc_ptr[s + 1]; ++q) {
                int li = pc->ownloc[q];
                y[dofs[li]] = z[li];
            }
            free(z);
        }
    } else {
        /* src/precond/asm.h:34-60: every overlap entry is added.  The
         * reference adds under omp critical in completion order; here the
         * solves run in parallel and the adds run in subdomain order, which
         * is the reference's order with one thread. */
        int np = pc->nparts;
        double** zs = (double**)malloc(sizeof(double*) * (size_t)np);
#pragma omp parallel for schedule(dynamic)
        for (int s = 0; s < np; ++s) {
            int ns = pc->sub_ptr[s + 1] - pc->sub_ptr[s];
            zs[s] = (double*)malloc(sizeof(double) * (size_t)(ns > 0 ? ns : 1));
            o_local_solve(pc, s, x, zs[s]);
        }
        for (int s = 0; s < np; ++s) {
            const int* dofs = pc->sub + pc->sub_ptr[s];
            int ns = pc->sub_ptr[s + 1] - pc->sub_ptr[s];
            for (int i = 0; i < ns; ++i) y[dofs[i]] += zs[s][i];
            free(zs[s]);
        }
        free(zs);
    }
}

void orc_pc_apply(const orc_pc* pc, const double* x, double* y, int n) {
    switch (pc->kind) {
    case ORC_PC_NONE:
        memcpy(y, x, sizeof(double) * (size_t)n);
        return;
    case ORC_PC_JACOBI: /* src/precond/jacobi.h:19-23 */
        for (int i = 0; i < n; ++i) y[i] = pc->inv_diag[i] * x[i];
        return;
    case ORC_PC_ILU0:
        orc_ilu0_solve(n, pc->ilu.rp, pc->ilu.ci, pc->ilu.lu, pc->ilu.diag, x, y);
        return;
    case ORC_PC_ASM:
    case ORC_PC_RAS:
        o_fine_apply(pc, x, y, n);
        return;
    default: {
        /* src/precond/two_level_schwarz.h:50-64 with the restriction and
         * prolongation of coarse_space.h:63-78 restricted to nonzeros. */
        double* zf = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
        o_fine_apply(pc, x, zf, n);
        int nc = pc->nc;
        double* r0 = (double*)malloc(sizeof(double) * (size_t)nc);
        double* z0 = (double*)malloc(sizeof(double) * (size_t)nc);
        for (int s = 0; s < nc; ++s) {
            double acc = 0.0;
            for (int q = pc->owned_ptr[s]; q < pc->owned_ptr[s + 1]; ++q)
                acc += pc->scale[s] * x[pc->owned[q]];
            r0[s] = acc;
        }
        o_coarse_solve(pc, r0, z0);
        /* z_coarse[k] = 0 + R0[s(k)][k] * z0[s(k)] */
        double* zc = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
        for (int s = 0; s < nc; ++s)
            for (int q = pc->owned_ptr[s]; q < pc->owned_ptr[s + 1]; ++q)
                zc[pc->owned[q]] += pc->scale[s] * z0[s];
        for (int i = 0; i < n; ++i) y[i] = zf[i] + zc[i];
        free(zf); free(r0); free(z0); free(zc);
        return;
    }
    }
}

int orc_pc_coarse(const orc_pc* pc, double* a0_out) {
    if (!pc->a0) return 0;
    if (a0_out) memcpy(a0_out, pc->a0, sizeof(double) * (size_t)pc->nc * (size_t)pc->nc);
    return pc->nc;
}

int orc_pc_sub_factor(const orc_pc* pc, int s, int* nnz_out, const int** rp,
                      const int** ci, const double** lu, const int** diag) {
    const o_ilu* f;
    if (pc->kind == ORC_PC_ILU0) f = &pc->ilu;
    else if (pc->loc && s >= 0 && s < pc->nparts) f = &pc->loc[s];
    else return -1;
    *nnz_out = f->nnz;
    *rp = f->rp; *ci = f->ci; *lu = f->lu; *diag = f->diag;
    return f->n;
}

void orc_pc_destroy(orc_pc* pc) {
    if (!pc) return;
    free(pc->inv_diag);
    if (pc->kind == ORC_PC_ILU0) o_ilu_free(&pc->ilu);
    if (pc->loc) {
        for (int s = 0; s < pc->nparts; ++s) o_ilu_free(&pc->loc[s]);
        free(pc->loc);
    }
    free(pc->owned_ptr); free(pc->owned); free(pc->sub_ptr); free(pc->sub);
    free(pc->ownloc_ptr); free(pc->ownloc);
    free(pc->scale); free(pc->a0); free(pc->lu0); free(pc->piv);
    free(pc);
}

/* ---------------------------------------------------------------- Krylov */
/* Givens rotation of src/core/gmres.cpp:9-30 (same as fgmres.cpp:10-24) */
typedef struct { double c, s; } o_rot;
static void o_rot_compute(o_rot* r, double a, double b) {
    if (fabs(b) < 1e-30) { r->c = 1.0; r->s = 0.0; }
    else if (fabs(b) > fabs(a)) {
        double t = -a / b;
        r->s = 1.0 / sqrt(1.0 + t * t);
        r->c = r->s * t;
    } else {
        double t = -b / a;
        r->c = 1.0 / sqrt(1.0 + t * t);
        r->s = r->c * t;
    }
}
static void o_rot_apply(const o_rot* r, double* h1, double* h2) {
    double t1 = r->c * *h1 - r->s * *h2;
    double t2 = r->s * *h1 + r->c * *h2;
    *h1 = t1;
    *h2 = t2;
}

/* src/core/gmres.cpp:34-160 */
int orc_gmres(int n, const int* rp, const int* ci, const double* v, const double* b,
              double* x, const orc_pc* pc, int m, int max_iter, double tol,
              int* iters, double* res_norm, double* hist, int hist_cap, int* hist_len) {
    size_t N = (size_t)(n > 0 ? n : 1);
    double* r = (double*)malloc(sizeof(double) * N);
    double* w = (double*)malloc(sizeof(double) * N);
    double* z = (double*)malloc(sizeof(double) * N);
    double* Av = (double*)malloc(sizeof(double) * N);
    double* V = (double*)malloc(sizeof(double) * N * (size_t)(m + 1));
    double* H = (double*)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
    double* g = (double*)calloc((size_t)(m + 1), sizeof(double));
    double* y = (double*)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    o_rot* rots = (o_rot*)calloc((size_t)(m > 0 ? m : 1), sizeof(o_rot));
    int total = 0, converged = 0, nh = 0;
    double last = 0.0;
    const int ld = m + 1;
    for (int cycle = 0; cycle < max_iter; ++cycle) {
        orc_spmv(n, rp, ci, v, x, r);
        for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
        if (pc && pc->kind != ORC_PC_NONE) orc_pc_apply(pc, r, z, n);
        else memcpy(z, r, sizeof(double) * N);
        double beta = o_norm2(z, n);
        if (beta < tol) { converged = 1; break; }
        for (int i = 0; i < n; ++i) V[i] = z[i] / beta;
        memset(H, 0, sizeof(double) * (size_t)(m + 1) * (size_t)m);
        memset(g, 0, sizeof(double) * (size_t)(m + 1));
        g[0] = beta;
        int j;
        for (j = 0; j < m; ++j) {
            double* vj = V + (size_t)j * N;
            orc_spmv(n, rp, ci, v, vj, Av);
            if (pc && pc->kind != ORC_PC_NONE) orc_pc_apply(pc, Av, w, n);
            else memcpy(w, Av, sizeof(double) * N);
            for (int i = 0; i <= j; ++i) {
                double h = o_dot(w, V + (size_t)i * N, n);
                H[i + j * ld] = h;
                o_axpy(-h, V + (size_t)i * N, w, n);
            }
            double hn = o_norm2(w, n);
            H[(j + 1) + j * ld] = hn;
            if (hn < 1e-30) { j++; break; }
            double* vn = V + (size_t)(j + 1) * N;
            for (int i = 0; i < n; ++i) vn[i] = w[i] / hn;
            for (int i = 0; i < j; ++i) o_rot_apply(&rots[i], &H[i + j * ld], &H[(i + 1) + j * ld]);
            o_rot_compute(&rots[j], H[j + j * ld], H[(j + 1) + j * ld]);
            o_rot_apply(&rots[j], &H[j + j * ld], &H[(j + 1) + j * ld]);
            o_rot_apply(&rots[j], &g[j], &g[j + 1]);
            double res = fabs(g[j + 1]);
            if (hist && nh < hist_cap) hist[nh] = res;
            nh++;
            last = res;
            total++;
            if (res < tol) { j++; converged = 1; break; }
        }
        int k = j;
        for (int i = k - 1; i >= 0; --i) {
            y[i] = g[i];
            for (int l = i + 1; l < k; ++l) y[i] -= H[i + l * ld] * y[l];
            y[i] /= H[i + i * ld];
        }
        for (int i = 0; i < k; ++i) o_axpy(y[i], V + (size_t)i * N, x, n);
        if (converged) break;
        if (total >= max_iter) break;
    }
    *iters = total;
    *res_norm = nh > 0 ? last : 0.0;
    if (hist_len) *hist_len = nh;
    free(r); free(w); free(z); free(Av); free(V); free(H); free(g); free(y); free(rots);
    return converged;
}

/* src/core/fgmres.cpp:28-144 */
int orc_fgmres(int n, const int* rp, const int* ci, const double* v, const double* b,
               double* x, const orc_pc* pc, int m, int max_iter, double tol,
               int* iters, double* res_norm, double* hist, int hist_cap, int* hist_len) {
    size_t N = (size_t)(n > 0 ? n : 1);
    double* V = (double*)calloc(N * (size_t)(m + 1), sizeof(double));
    double* Z = (double*)calloc(N * (size_t)(m > 0 ? m : 1), sizeof(double));
    double* H = (double*)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
    double* g = (double*)calloc((size_t)(m + 1), sizeof(double));
    double* y = (double*)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
    o_rot* rots = (o_rot*)calloc((size_t)(m > 0 ? m : 1), sizeof(o_rot));
    for (int i = 0; i < m; ++i) { rots[i].c = 1.0; rots[i].s = 0.0; }
    double* r = (double*)malloc(sizeof(double) * N);
    double* w = (double*)malloc(sizeof(double) * N);
    int total = 0, converged = 0, nh = 0;
    double last = 0.0;
    const int ld = m + 1;
    for (int cycle = 0; cycle < max_iter; ++cycle) {
        orc_spmv(n, rp, ci, v, x, r);
        for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
        double beta = o_norm2(r, n);
        if (beta < tol) { converged = 1; break; }
        double inv_beta = 1.0 / beta;
        for (int i = 0; i < n; ++i) V[i] = r[i] * inv_beta;
        memset(H, 0, sizeof(double) * (size_t)(m + 1) * (size_t)m);
        memset(g, 0, sizeof(double) * (size_t)(m + 1));
        g[0] = beta;
        int j;
        for (j = 0; j < m; ++j) {
            double* vj = V + (size_t)j * N;
            double* zj = Z + (size_t)j * N;
            if (pc && pc->kind != ORC_PC_NONE) orc_pc_apply(pc, vj, zj, n);
            else memcpy(zj, vj, sizeof(double) * N);
            orc_spmv(n, rp, ci, v, zj, w);
            for (int i = 0; i <= j; ++i) {
                double h = o_dot(w, V + (size_t)i * N, n);
                H[i + j * ld] = h;
                o_axpy(-h, V + (size_t)i * N, w, n);
            }
            double hn = o_norm2(w, n);
            H[(j + 1) + j * ld] = hn;
            if (hn < 1e-30) { j++; break; }
            double inv_h = 1.0 / hn;
            double* vn = V + (size_t)(j + 1) * N;
            for (int i = 0; i < n; ++i) vn[i] = w[i] * inv_h;
            for (int i = 0; i < j; ++i) o_rot_apply(&rots[i], &H[i + j * ld], &H[(i + 1) + j * ld]);
            o_rot_compute(&rots[j], H[j + j * ld], H[(j + 1) + j * ld]);
            o_rot_apply(&rots[j], &H[j + j * ld], &H[(j + 1) + j * ld]);
            o_rot_apply(&rots[j], &g[j], &g[j + 1]);
            double res = fabs(g[j + 1]);
            if (hist && nh < hist_cap) hist[nh] = res;
            nh++;
            last = res;
            total++;
            if (res < tol) { j++; converged = 1; break; }
        }
        int k = j;
        for (int i = k - 1; i >= 0; --i) {
            y[i] = g[i];
            for (int l = i + 1; l < k; ++l) y[i] -= H[i + l * ld] * y[l];
            y[i] /= H[i + i * ld];
        }
        for (int i = 0; i < k; ++i) o_axpy(y[i], Z + (size_t)i * N, x, n);
        if (converged) break;
        if (total >= max_iter) break;
    }
    *iters = total;
    *res_norm = nh > 0 ? last : 0.0;
    if (hist_len) *hist_len = nh;
    free(V); free(Z); free(H); free(g); free(y); free(rots); free(r); free(w);
    return converged;
}

/* ---------------------------------------------------------------- generators */
/* src/mesh/poisson.h:10-38: row-major idx = iy*nx+ix, entries in ascending
 * column order (south, west, centre, east, north), 4 / -1. */
int orc_poisson2d(int nx, int ny, int* rp, int* ci, double* v) {
    int nz = 0;
    for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix) {
            int idx = iy * nx + ix;
            if (rp) rp[idx] = nz;
#define PUT(c, val) do { if (ci) { ci[nz] = (c); v[nz] = (val); } ++nz; } while (0)
            if (iy > 0) PUT(idx - nx, -1.0);
            if (ix > 0) PUT(idx - 1, -1.0);
            PUT(idx, 4.0);
            if (ix < nx - 1) PUT(idx + 1, -1.0);
            if (iy < ny - 1) PUT(idx + nx, -1.0);
        }
    if (rp) rp[nx * ny] = nz;
    return nz;
}

/* src/mesh/poisson.h:41-74: idx = iz*nx*ny + iy*nx + ix, 6 / -1. */
int orc_poisson3d(int nx, int ny, int nz_, int* rp, int* ci, double* v) {
    int nz = 0, nxy = nx * ny;
    for (int iz = 0; iz < nz_; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                int idx = iz * nxy + iy * nx + ix;
                if (rp) rp[idx] = nz;
                if (iz > 0) PUT(idx - nxy, -1.0);
                if (iy > 0) PUT(idx - nx, -1.0);
                if (ix > 0) PUT(idx - 1, -1.0);
                PUT(idx, 6.0);
                if (ix < nx - 1) PUT(idx + 1, -1.0);
                if (iy < ny - 1) PUT(idx + nx, -1.0);
                if (iz < nz_ - 1) PUT(idx + nxy, -1.0);
            }
#undef PUT
    if (rp) rp[nxy * nz_] = nz;
    return nz;
}

/* ------------------------------------------------------------------------
 * Benchmark inputs (no reference counterpart).  The project generates its
 * 3D variable-coefficient operator, uneven box partitions and uniform
 * vectors itself (the package's sg_gen_varcoef3d, sg_partition_boxes,
 * sg_gen_uniform); they are restated here so that the CPU baseline builds
 * the same problem without loading the package.  tests/test_oracle_inputs.py
 * checks them against the package bit for bit.  Compiled like the rest of
 * this file with -ffp-contract=off, as the package's host code is.
 * ---------------------------------------------------------------------- */
static uint64_t orc_next64(uint64_t* state) {
    /* SplitMix64 (Steele, Lea, Flood 2014) */
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double orc_unit(uint64_t* state) {
    return (double)(orc_next64(state) >> 11) * (1.0 / 9007199254740992.0); /* 2^-53 */
}

void orc_uniform(uint64_t seed, int n, double lo, double hi, double* out) {
    uint64_t st = seed;
    for (int i = 0; i < n; ++i) out[i] = lo + (hi - lo) * orc_unit(&st);
}

/* Recursive coordinate bisection into nparts boxes: a box of k parts is cut
 * across its longest axis (x, then y, then z on ties) at the fraction
 * k1/k * (1 + spread * (2u - 1)) of its length (k1 = k/2, u uniform from the
 * seeded stream, one draw per cut), clamped to leave both halves non-empty;
 * the lower half takes parts [base, base+k1) and is cut next (depth first). */
int orc_partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed,
                        int* part) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || nparts < 1) return 1;
    typedef struct { int lo[3], hi[3], k, base; } box_t;
    box_t* todo = (box_t*)malloc(sizeof(box_t) * (size_t)(2 * nparts + 2));
    if (!todo) return 3;
    int top = 0;
    box_t root = {{0, 0, 0}, {nx, ny, nz}, nparts, 0};
    todo[top++] = root;
    uint64_t st = seed;
    while (top > 0) {
        box_t bx = todo[--top];
        if (bx.k == 1) {
            for (int z = bx.lo[2]; z < bx.hi[2]; ++z)
                for (int y = bx.lo[1]; y < bx.hi[1]; ++y)
                    for (int x = bx.lo[0]; x < bx.hi[0]; ++x)
                        part[((size_t)z * ny + y) * nx + x] = bx.base;
            continue;
        }
        int ax = 0;
        for (int d = 1; d < 3; ++d)
            if (bx.hi[d] - bx.lo[d] > bx.hi[ax] - bx.lo[ax]) ax = d;
        const int len = bx.hi[ax] - bx.lo[ax];
        if (len < 2) {
            free(todo);
            return 2;
        }
        const int k1 = bx.k / 2;
        const double frac = (double)k1 / bx.k * (1.0 + spread * (2.0 * orc_unit(&st) - 1.0));
        long cut = lround(frac * len);
        if (cut < 1) cut = 1;
        if (cut > len - 1) cut = len - 1;
        box_t lower = bx, upper = bx;
        lower.k = k1;
        lower.hi[ax] = bx.lo[ax] + (int)cut;
        upper.k = bx.k - k1;
        upper.base = bx.base + k1;
        upper.lo[ax] = bx.lo[ax] + (int)cut;
        todo[top++] = upper;
        todo[top++] = lower;
    }
    free(todo);
    return 0;
}

/* ln k of the benchmark's coefficient field, then k = exp(sigma * g):
 * g is Gaussian white noise (Box-Muller on the seeded stream, two values per
 * pair of draws) on the grid padded by R = ceil(3 corr / sqrt 2) cells per
 * side, smoothed by the separable kernel exp(-d^2 / corr^2) along x, y and z
 * in turn, then standardised to zero mean and unit sample variance. */
static double* orc_coef_field(int nx, int ny, int nz, double sigma, double corr, uint64_t seed) {
    const int R = (int)fmax(1.0, ceil(3.0 * (corr / sqrt(2.0))));
    const int W = 2 * R + 1;
    double* ker = (double*)malloc(sizeof(double) * (size_t)W);
    for (int d = -R; d <= R; ++d) ker[d + R] = exp(-(double)d * d / (corr * corr));
    const size_t px = (size_t)nx + 2 * R, py = (size_t)ny + 2 * R, pz = (size_t)nz + 2 * R;
    const size_t npad = px * py * pz, n = (size_t)nx * ny * nz;
    double* noise = (double*)malloc(sizeof(double) * npad);
    uint64_t st = seed;
    const double two_pi = 6.283185307179586232; /* 2 * M_PI, as the double product */
    for (size_t i = 0; i < npad; i += 2) {
        const double u1 = 1.0 - orc_unit(&st), u2 = orc_unit(&st);
        const double rad = sqrt(-2.0 * log(u1));
        noise[i] = rad * cos(two_pi * u2);
        if (i + 1 < npad) noise[i + 1] = rad * sin(two_pi * u2);
    }
    /* smooth along x (padded y, z kept), then y, then z */
    double* sx = (double*)malloc(sizeof(double) * (size_t)nx * py * pz);
    for (size_t z = 0; z < pz; ++z)
        for (size_t y = 0; y < py; ++y)
            for (int x = 0; x < nx; ++x) {
                const double* src = noise + (z * py + y) * px + x;
                double acc = 0.0;
                for (int d = 0; d < W; ++d) acc += ker[d] * src[d];
                sx[(z * py + y) * nx + x] = acc;
            }
    free(noise);
    double* sy = (double*)malloc(sizeof(double) * (size_t)nx * ny * pz);
    for (size_t z = 0; z < pz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                double acc = 0.0;
                for (int d = 0; d < W; ++d) acc += ker[d] * sx[(z * py + y + d) * nx + x];
                sy[(z * ny + y) * nx + x] = acc;
            }
    free(sx);
    double* g = (double*)malloc(sizeof(double) * n);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                double acc = 0.0;
                for (int d = 0; d < W; ++d)
                    acc += ker[d] * sy[(((size_t)z + d) * ny + y) * nx + x];
                g[((size_t)z * ny + y) * nx + x] = acc;
            }
    free(sy);
    free(ker);
    double mean = 0.0;
    for (size_t i = 0; i < n; ++i) mean += g[i];
    mean /= (double)n;
    double var = 0.0;
    for (size_t i = 0; i < n; ++i) var += (g[i] - mean) * (g[i] - mean);
    var /= (double)n;
    const double inv = var > 0 ? 1.0 / sqrt(var) : 1.0;
    for (size_t i = 0; i < n; ++i) g[i] = exp(sigma * (g[i] - mean) * inv);
    return g;
}

/* -div(k grad u), 7-point, Dirichlet: the coupling across an interior face
 * is the harmonic mean 2 k_a k_b / (k_a + k_b) of the two cells, a boundary
 * face couples to the zero boundary value with the cell's own k, and the
 * diagonal is the sum of the six face coefficients (added -z, -y, -x, +x,
 * +y, +z).  Rows and columns in make_poisson_3d's order
 * (src/mesh/poisson.h:42-74).  Returns nnz; rp == NULL only sizes. */
int orc_varcoef3d(int nx, int ny, int nz, double sigma, double corr, uint64_t seed, int* rp,
                  int* ci, double* v) {
    if (!rp) return orc_poisson3d(nx, ny, nz, NULL, NULL, NULL);
    double* k = orc_coef_field(nx, ny, nz, sigma, corr, seed);
    const int nxy = nx * ny;
    int e = 0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                const int c = iz * nxy + iy * nx + ix;
                const double kc = k[c];
#define ORC_FACE(nb) (2.0 * kc * k[nb] / (kc + k[nb]))
                const double f[6] = {iz > 0 ? ORC_FACE(c - nxy) : kc,
                                     iy > 0 ? ORC_FACE(c - nx) : kc,
                                     ix > 0 ? ORC_FACE(c - 1) : kc,
                                     ix < nx - 1 ? ORC_FACE(c + 1) : kc,
                                     iy < ny - 1 ? ORC_FACE(c + nx) : kc,
                                     iz < nz - 1 ? ORC_FACE(c + nxy) : kc};
#undef ORC_FACE
                const double diag = f[0] + f[1] + f[2] + f[3] + f[4] + f[5];
                rp[c] = e;
                if (iz > 0) { ci[e] = c - nxy; v[e++] = -f[0]; }
                if (iy > 0) { ci[e] = c - nx; v[e++] = -f[1]; }
                if (ix > 0) { ci[e] = c - 1; v[e++] = -f[2]; }
                ci[e] = c; v[e++] = diag;
                if (ix < nx - 1) { ci[e] = c + 1; v[e++] = -f[3]; }
                if (iy < ny - 1) { ci[e] = c + nx; v[e++] = -f[4]; }
                if (iz < nz - 1) { ci[e] = c + nxy; v[e++] = -f[5]; }
            }
    rp[nxy * nz] = e;
    free(k);
    return e;
}

/* ------------------------------------------------------------------------
 * BiCGSTAB with right preconditioning (src/core/bicgstab.h:57-204), in the
 * reference's operation order.  Returns the converged flag; iters, res_norm
 * and the history of ||r|| (or ||s|| on an early exit) as the reference's
 * GMRESResult holds them.
 * ---------------------------------------------------------------------- */
int orc_bicgstab(int n, const int* rp, const int* ci, const double* v, const double* b,
                 double* x, const orc_pc* pc, int max_iter, double tol, int* iters,
                 double* res_norm, double* hist, int hist_cap, int* hist_len) {
    const size_t bytes = sizeof(double) * (size_t)(n > 0 ? n : 1);
    double *r = malloc(bytes), *rh = malloc(bytes), *p = calloc((size_t)(n > 0 ? n : 1), 8),
           *vv = calloc((size_t)(n > 0 ? n : 1), 8), *y = malloc(bytes), *z = malloc(bytes),
           *s = malloc(bytes), *t = malloc(bytes), *tmp = malloc(bytes);
    int nh = 0, conv = 0, it_out = 0;
    double res = 0.0;
#define O_HIST(val) do { if (hist && nh < hist_cap) hist[nh] = (val); ++nh; } while (0)
#define O_PREC(in, out) do { if (pc) orc_pc_apply(pc, in, out, n); \
                             else memcpy(out, in, sizeof(double) * (size_t)n); } while (0)
    orc_spmv(n, rp, ci, v, x, tmp); /* bicgstab.h:76-78 */
    for (int i = 0; i < n; ++i) r[i] = b[i] - tmp[i];
    memcpy(rh, r, sizeof(double) * (size_t)n);
    const double r0 = o_norm2(r, n);
    if (r0 < 1e-14) { /* :83-88 */
        conv = 1;
        res = r0;
        goto done;
    }
    double rho = 1.0, alpha = 1.0, omega = 1.0, rho_prev;
    for (int iter = 1; iter <= max_iter; ++iter) {
        rho_prev = rho;
        rho = o_dot(rh, r, n);
        if (fabs(rho) < 1e-300) { /* :101-107 */
            it_out = iter;
            res = o_norm2(r, n);
            conv = 0;
            break;
        }
        if (iter == 1) {
            memcpy(p, r, sizeof(double) * (size_t)n);
        } else {
            const double beta = (rho / rho_prev) * (alpha / omega);
            for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * vv[i]);
        }
        O_PREC(p, y);
        orc_spmv(n, rp, ci, v, y, vv);
        const double rhv = o_dot(rh, vv, n);
        if (fabs(rhv) < 1e-300) { /* :125-130 */
            it_out = iter;
            res = o_norm2(r, n);
            conv = 0;
            break;
        }
        alpha = rho / rhv;
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * vv[i];
        const double sn = o_norm2(s, n);
        if (sn < tol * r0) { /* :140-148 lucky exit after the half step */
            for (int i = 0; i < n; ++i) x[i] += alpha * y[i];
            it_out = iter;
            res = sn;
            conv = 1;
            O_HIST(sn);
            break;
        }
        O_PREC(s, z);
        orc_spmv(n, rp, ci, v, z, t);
        const double tt = o_dot(t, t, n);
        if (tt < 1e-300) { /* :158-165 */
            for (int i = 0; i < n; ++i) x[i] += alpha * y[i];
            it_out = iter;
            res = sn;
            conv = sn < tol * r0;
            break;
        }
        omega = o_dot(t, s, n) / tt;
        for (int i = 0; i < n; ++i) x[i] += alpha * y[i] + omega * z[i];
        for (int i = 0; i < n; ++i) r[i] = s[i] - omega * t[i];
        const double rn = o_norm2(r, n);
        O_HIST(rn);
        it_out = iter;
        res = rn;
        conv = 0;
        if (rn < tol * r0) { /* :181-186 */
            conv = 1;
            break;
        }
        if (fabs(omega) < 1e-300) break; /* :188-194 stagnation */
    }
done:
#undef O_HIST
#undef O_PREC
    *iters = it_out;
    *res_norm = res;
    if (hist_len) *hist_len = nh;
    free(r); free(rh); free(p); free(vv); free(y); free(z); free(s); free(t); free(tmp);
    return conv;
}

/* ------------------------------------------------------------------------
 * Analysis tools (src/analysis/condition_estimator.h:94-191,
 * src/analysis/spectral_analysis.h:30-97).
 * ---------------------------------------------------------------------- */
/* the reference's start vector: a 32-bit LCG (x <- 1664525 x + 1013904223)
 * read as a signed int / 2^31, normalised (condition_estimator.h:107-117) */
static void o_lcg_unit(int n, unsigned seed, double* v, int guard_tiny) {
    unsigned st = seed;
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) {
        st = st * 1664525u + 1013904223u;
        v[i] = (double)(int)st / 2147483648.0;
        nrm += v[i] * v[i];
    }
    nrm = sqrt(nrm);
    if (guard_tiny && nrm < 1e-14) nrm = 1.0;
    for (int i = 0; i < n; ++i) v[i] /= nrm;
}

static int o_cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* eigenvalues of the symmetric tridiagonal (d, e) by implicit QL with the
 * Wilkinson shift, as tridiag_eigs_ql (condition_estimator.h:42-88) runs it
 * (including its handling of an exactly zero rotation radius); sorted */
static void o_tridiag_eigs(double* d, double* e, int n) {
    const int max_iter = 100 * n;
    for (int l = 0; l < n; ++l) {
        int m, iter = 0;
        do {
            for (m = l; m < n - 1; ++m) {
                const double off = fabs(d[m]) + fabs(d[m + 1]);
                if (fabs(e[m]) <= 1e-14 * off) break;
            }
            if (m == l) break;
            if (++iter > max_iter) break;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            for (int i = m - 1; i >= l; --i) {
                const double f = s * e[i];
                const double bb = c * e[i];
                r = hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= p;
                    e[m] = 0.0;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * bb;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - bb;
            }
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        } while (m != l);
    }
    qsort(d, (size_t)n, sizeof(double), o_cmp_double);
}

/* estimate_condition: k Lanczos steps on M^{-1}A (A when pc is NULL or of
 * kind NONE), extreme Ritz values of the tridiagonal.  out: lambda_min,
 * lambda_max, kappa; iout: steps, valid.  Returns the steps (0: no estimate). */
int orc_condition(int n, const int* rp, const int* ci, const double* v, const orc_pc* pc, int k,
                  unsigned seed, double* out, int* iout) {
    out[0] = out[1] = out[2] = 0.0;
    iout[0] = iout[1] = 0;
    if (k > n) k = n;
    if (k < 2) return 0;
    const size_t bytes = sizeof(double) * (size_t)n;
    double *vc = malloc(bytes), *vp = calloc((size_t)n, 8), *w = malloc(bytes), *z = malloc(bytes);
    double* al = malloc(sizeof(double) * (size_t)k);
    double* be = calloc((size_t)k + 1, sizeof(double));
    o_lcg_unit(n, seed, vc, 1);
    int na = 0, nb = 0;
    double beta = 0.0;
    for (int j = 0; j < k; ++j) {
        orc_spmv(n, rp, ci, v, vc, w);
        if (pc) orc_pc_apply(pc, w, z, n);
        else memcpy(z, w, bytes);
        const double alpha = o_dot(vc, z, n);
        al[na++] = alpha;
        for (int i = 0; i < n; ++i) z[i] -= alpha * vc[i] + beta * vp[i];
        const double bn = o_norm2(z, n);
        if (bn < 1e-10 * (1.0 + fabs(alpha))) break;
        if (j < k - 1) {
            be[nb++] = bn;
            memcpy(vp, vc, bytes);
            beta = bn;
            const double inv = 1.0 / bn;
            for (int i = 0; i < n; ++i) vc[i] = z[i] * inv;
        }
    }
    int steps = 0;
    int finite = 1;
    for (int i = 0; i < na; ++i) finite &= isfinite(al[i]) != 0;
    for (int i = 0; i < nb; ++i) finite &= isfinite(be[i]) != 0;
    if (na >= 2 && finite) {
        for (int i = nb; i < na; ++i) be[i] = 0.0;
        o_tridiag_eigs(al, be, na);
        int lo = -1, hi = -1;
        for (int i = 0; i < na; ++i)
            if (isfinite(al[i])) {
                if (lo < 0) lo = i;
                hi = i;
            }
        if (lo >= 0) {
            out[0] = al[lo];
            out[1] = al[hi];
            out[2] = fabs(al[lo]) > 1e-14 ? al[hi] / al[lo] : 1e30;
            iout[0] = steps = na;
            iout[1] = al[lo] > 0.0;
        }
    }
    free(vc); free(vp); free(w); free(z); free(al); free(be);
    return steps;
}

/* estimate_spectral_radius: power iteration on E = I - M^{-1}A, stopping
 * when the Rayleigh quotient changes by < tol (1 + |mu|); reports |mu| of
 * the step before the last, as the reference does.  out: rho; iout: steps,
 * rho < 1. */
void orc_spectral(int n, const int* rp, const int* ci, const double* v, const orc_pc* pc,
                  int max_iter, double tol, unsigned seed, double* out, int* iout) {
    const size_t bytes = sizeof(double) * (size_t)(n > 0 ? n : 1);
    double *vv = malloc(bytes), *w = malloc(bytes), *z = malloc(bytes);
    o_lcg_unit(n, seed, vv, 0);
    double mu_prev = 0.0;
    int steps = 0;
    for (int it = 0; it < max_iter; ++it) {
        orc_spmv(n, rp, ci, v, vv, w);
        if (pc) orc_pc_apply(pc, w, z, n);
        else memcpy(z, w, bytes);
        for (int i = 0; i < n; ++i) w[i] = vv[i] - z[i];
        double mu = o_dot(vv, w, n);
        const double en = o_norm2(w, n);
        if (en < 1e-14) {
            steps = it + 1;
            mu = 0.0;
            break;
        }
        for (int i = 0; i < n; ++i) vv[i] = w[i] / en;
        steps = it + 1;
        if (fabs(mu - mu_prev) < tol * (1.0 + fabs(mu))) break;
        mu_prev = mu;
    }
    out[0] = fabs(mu_prev);
    iout[0] = steps;
    iout[1] = out[0] < 1.0;
    free(vv); free(w); free(z);
}
