/*
 * dfg_oracle.c -- CPU oracle (test infrastructure only; see dfg_oracle.h).
 *
 * A plain-C restatement of DelFEM's FE assembly, Dirichlet finalize, block
 * ILU(0) and PCG, written to reproduce the reference's floating-point
 * operation order so results are bit-identical to the reference compiled
 * with the same flags (-O2 -ffp-contract=off).  Each function cites the
 * reference file:line it restates.  Only tests/, smoke() and bench.py's
 * CPU baseline use this file.
 */
#include "dfg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

double dfo_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------------------------ */
/* Pattern                                                                   */
/* ------------------------------------------------------------------------ */

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* Elements-surrounding-point, then point-surrounding-point excluding self,
 * sorted ascending: the result of CElemAry::MakePattern_FEM
 * (femfield/elem_ary.cpp:225-245, crs.Sort()). */
long dfo_pattern(int nnode, int nelem, int nnoel, const int* conn,
                 int* rowptr, int* colind) {
  if (nnode < 0 || nelem < 0 || nnoel < 1) return -1;
  int* esup_ptr = (int*)calloc((size_t)nnode + 1, sizeof(int));
  for (long e = 0; e < nelem; ++e)
    for (int k = 0; k < nnoel; ++k) {
      int v = conn[e * nnoel + k];
      if (v < 0 || v >= nnode) { free(esup_ptr); return -1; }
      esup_ptr[v + 1]++;
    }
  for (int i = 0; i < nnode; ++i) esup_ptr[i + 1] += esup_ptr[i];
  int* esup = (int*)malloc(sizeof(int) * (size_t)(esup_ptr[nnode] + 1));
  int* fill = (int*)malloc(sizeof(int) * ((size_t)nnode + 1));
  memcpy(fill, esup_ptr, sizeof(int) * (size_t)nnode);
  for (long e = 0; e < nelem; ++e)
    for (int k = 0; k < nnoel; ++k) esup[fill[conn[e * nnoel + k]]++] = (int)e;
  int* mark = (int*)malloc(sizeof(int) * ((size_t)nnode + 1));
  for (int i = 0; i < nnode; ++i) mark[i] = -1;
  long nnz = 0;
  int* tmp = (int*)malloc(sizeof(int) * ((size_t)nnode + 1));
  if (rowptr) rowptr[0] = 0;
  for (int i = 0; i < nnode; ++i) {
    int cnt = 0;
    for (int p = esup_ptr[i]; p < esup_ptr[i + 1]; ++p) {
      int e = esup[p];
      for (int k = 0; k < nnoel; ++k) {
        int j = conn[(long)e * nnoel + k];
        if (j == i || mark[j] == i) continue;
        mark[j] = i;
        tmp[cnt++] = j;
      }
    }
    if (colind) {
      qsort(tmp, (size_t)cnt, sizeof(int), cmp_int);
      memcpy(colind + nnz, tmp, sizeof(int) * (size_t)cnt);
    }
    nnz += cnt;
    if (rowptr) rowptr[i + 1] = (int)nnz;
  }
  free(tmp); free(mark); free(fill); free(esup); free(esup_ptr);
  return nnz;
}

/* matvec/matdiafrac_blkcrs.cpp:203-218 */
void dfo_diaind(int n, const int* rowptr, const int* colind, int* diaind) {
  for (int i = 0; i < n; ++i) {
    diaind[i] = rowptr[i + 1];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
      if (colind[c] > i) { diaind[i] = c; break; }
  }
}

/* ------------------------------------------------------------------------ */
/* ILU(k) fill pattern -- CMatDiaFrac_BlkCrs::AddFracPtn                      */
/* (matvec/matdiafrac_blkcrs.cpp:1254-1382) as CPreconditioner_ILU calls it   */
/* for one segment (ls/preconditioner.cpp:96-157)                             */
/* ------------------------------------------------------------------------ */

/* Row i starts as the sorted columns of A's row i, all at level 0.  Its
 * entries k < i are visited in ascending order, fill entries found on the way
 * included; an entry of level L >= lev_fill (any level when lev_fill == -1
 * is allowed) spawns nothing.  Entry k spawns, for every entry (k, j), j > k,
 * of the finished row k whose level M is below the limit, the entry (i, j) at
 * level max(L, M) + 1 unless (i, j) is already in the row (its level then
 * stays as it is) or j == i.  Unchanged pattern for lev_fill == 0, an empty
 * off-diagonal pattern, or a full one.  Returns nnz of the factor; when it
 * exceeds cap nothing is written and the caller retries with that capacity. */
long dfo_ilu_pattern(int n, const int* rowptr, const int* colind, int lev_fill,
                     int* rowptr_f, int* colind_f, long cap) {
  const long nnz = rowptr[n];
  if (lev_fill == 0 || nnz == 0 || nnz == (long)n * (n - 1)) {
    if (nnz > cap) return nnz;
    memcpy(rowptr_f, rowptr, sizeof(int) * (size_t)(n + 1));
    memcpy(colind_f, colind, sizeof(int) * (size_t)nnz);
    return nnz;
  }
  const int END = n;                     /* list terminator */
  int* nxt = (int*)malloc(sizeof(int) * (size_t)(n + 1));  /* nxt[n] = head */
  int* lv = (int*)malloc(sizeof(int) * (size_t)n);
  int* mark = (int*)malloc(sizeof(int) * (size_t)n);
  int* dia = (int*)malloc(sizeof(int) * (size_t)n);
  long fcap = nnz * 2 + 16, fz = 0;
  int* fcol = (int*)malloc(sizeof(int) * (size_t)fcap);
  int* flev = (int*)malloc(sizeof(int) * (size_t)fcap);
  long* fptr = (long*)malloc(sizeof(long) * (size_t)(n + 1));
  for (int i = 0; i < n; ++i) mark[i] = -1;
  fptr[0] = 0;
  for (int i = 0; i < n; ++i) {
    /* the row as a sorted linked list; nxt[END] is its first column */
    int last = END;
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      const int j = colind[c];
      nxt[last] = j;
      lv[j] = 0;
      mark[j] = i;
      last = j;
    }
    nxt[last] = END;
    for (int k = nxt[END]; k != END; k = nxt[k]) {
      const int lik = lv[k];
      if (lev_fill != -1 && lik + 1 > lev_fill) continue;
      if (k >= i) break;
      int pos = k; /* insertion point search starts at k: every new column is > k */
      for (long kj = dia[k]; kj < fptr[k + 1]; ++kj) {
        const int lkj = flev[kj];
        if (lev_fill != -1 && lkj + 1 > lev_fill) continue;
        const int j = fcol[kj];
        if (j == i || mark[j] == i) continue;
        while (nxt[pos] != END && nxt[pos] < j) pos = nxt[pos];
        nxt[j] = nxt[pos];
        nxt[pos] = j;
        lv[j] = (lik > lkj ? lik : lkj) + 1;
        mark[j] = i;
        pos = j;
      }
    }
    /* emit the row */
    int cnt = 0;
    for (int j = nxt[END]; j != END; j = nxt[j]) ++cnt;
    if (fz + cnt > fcap) {
      while (fz + cnt > fcap) fcap *= 2;
      fcol = (int*)realloc(fcol, sizeof(int) * (size_t)fcap);
      flev = (int*)realloc(flev, sizeof(int) * (size_t)fcap);
    }
    dia[i] = -1;
    for (int j = nxt[END]; j != END; j = nxt[j]) {
      if (dia[i] < 0 && j > i) dia[i] = (int)fz;
      fcol[fz] = j;
      flev[fz] = lv[j];
      ++fz;
    }
    if (dia[i] < 0) dia[i] = (int)fz;
    fptr[i + 1] = fz;
  }
  if (fz <= cap) {
    for (int i = 0; i <= n; ++i) rowptr_f[i] = (int)fptr[i];
    memcpy(colind_f, fcol, sizeof(int) * (size_t)fz);
  }
  free(nxt); free(lv); free(mark); free(dia); free(fcol); free(flev); free(fptr);
  return fz;
}

/* SetValue_Initialize (matvec/matdiafrac_blkcrs.h:90-96): the factor storage
 * is zeroed, then A's diagonal and off-diagonal blocks are copied into the
 * slots of the same columns (A's pattern is a subset of the factor's). */
int dfo_ilu_init(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                 const int* rowptr_f, const int* colind_f, double* fdiag, double* foffd) {
  const int bs = b * b;
  memcpy(fdiag, diag, sizeof(double) * (size_t)n * bs);
  memset(foffd, 0, sizeof(double) * (size_t)rowptr_f[n] * bs);
  for (int i = 0; i < n; ++i) {
    int cf = rowptr_f[i];
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      while (cf < rowptr_f[i + 1] && colind_f[cf] < colind[c]) ++cf;
      if (cf == rowptr_f[i + 1] || colind_f[cf] != colind[c]) return -1;
      memcpy(foffd + (size_t)cf * bs, offd + (size_t)c * bs, sizeof(double) * bs);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Scatter (Mearge) -- matvec/matdia_blkcrs.cpp:165-258                      */
/* ------------------------------------------------------------------------ */

typedef struct {
  int n, b;
  const int* rowptr;
  const int* colind;
  double* diag;
  double* offd;
  int* marker; /* column -> CRS slot for the row being merged, -1 otherwise */
} Merger;

static void merger_init(Merger* m, int n, int b, const int* rowptr, const int* colind,
                        double* diag, double* offd) {
  m->n = n; m->b = b; m->rowptr = rowptr; m->colind = colind;
  m->diag = diag; m->offd = offd;
  m->marker = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  for (int i = 0; i < n; ++i) m->marker[i] = -1;
}
static void merger_free(Merger* m) { free(m->marker); }

/* emat[(i*nno+j)*bs + idof*b + jdof], nodes no[0..nno) */
static void merge(Merger* m, int nno, const int* no, const double* emat) {
  const int bs = m->b * m->b;
  for (int i = 0; i < nno; ++i) {
    const int ib = no[i];
    for (int c = m->rowptr[ib]; c < m->rowptr[ib + 1]; ++c) m->marker[m->colind[c]] = c;
    for (int j = 0; j < nno; ++j) {
      const double* pin = &emat[(i * nno + j) * bs];
      if (i == j) {
        double* pout = &m->diag[(long)ib * bs];
        for (int k = 0; k < bs; ++k) pout[k] += pin[k];
      } else {
        const int slot = m->marker[no[j]];
        if (slot == -1) continue;
        double* pout = &m->offd[(long)slot * bs];
        for (int k = 0; k < bs; ++k) pout[k] += pin[k];
      }
    }
    for (int c = m->rowptr[ib]; c < m->rowptr[ib + 1]; ++c) m->marker[m->colind[c]] = -1;
  }
}

/* ------------------------------------------------------------------------ */
/* Shape-function kernels                                                    */
/* ------------------------------------------------------------------------ */

/* femeqn/ker_emat_tri.cpp:13-15 */
static double tri_area(const double* p0, const double* p1, const double* p2) {
  return 0.5 * ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]));
}

/* femeqn/ker_emat_tri.cpp:36-69 (the constant terms are not needed) */
static void tri_dldx(double dldx[3][2], const double* p0, const double* p1, const double* p2) {
  const double area = tri_area(p0, p1, p2);
  const double tmp1 = 0.5 / area;
  dldx[0][0] = tmp1 * (p1[1] - p2[1]);
  dldx[1][0] = tmp1 * (p2[1] - p0[1]);
  dldx[2][0] = tmp1 * (p0[1] - p1[1]);
  dldx[0][1] = tmp1 * (p2[0] - p1[0]);
  dldx[1][1] = tmp1 * (p0[0] - p2[0]);
  dldx[2][1] = tmp1 * (p1[0] - p0[0]);
}

/* include/delfem/femeqn/ker_emat_tet.h:32-39 (note the truncated 1/6 literal) */
static double tet_volume(const double* p0, const double* p1, const double* p2, const double* p3) {
  double vol = (p1[0] - p0[0]) * ((p2[1] - p0[1]) * (p3[2] - p0[2]) - (p3[1] - p0[1]) * (p2[2] - p0[2]))
             - (p1[1] - p0[1]) * ((p2[0] - p0[0]) * (p3[2] - p0[2]) - (p3[0] - p0[0]) * (p2[2] - p0[2]))
             + (p1[2] - p0[2]) * ((p2[0] - p0[0]) * (p3[1] - p0[1]) - (p3[0] - p0[0]) * (p2[1] - p0[1]));
  vol *= 0.1666666666666;
  return vol;
}

/* include/delfem/femeqn/ker_emat_tet.h:42-77 */
static void tet_dldx(double d[4][3], const double* p0, const double* p1, const double* p2, const double* p3) {
  const double vol = tet_volume(p0, p1, p2, p3);
  const double t = 1.0 / (vol * 6.0);
  d[0][0] = -t * ((p2[1] - p1[1]) * (p3[2] - p1[2]) - (p3[1] - p1[1]) * (p2[2] - p1[2]));
  d[0][1] = +t * ((p2[0] - p1[0]) * (p3[2] - p1[2]) - (p3[0] - p1[0]) * (p2[2] - p1[2]));
  d[0][2] = -t * ((p2[0] - p1[0]) * (p3[1] - p1[1]) - (p3[0] - p1[0]) * (p2[1] - p1[1]));
  d[1][0] = +t * ((p3[1] - p2[1]) * (p0[2] - p2[2]) - (p0[1] - p2[1]) * (p3[2] - p2[2]));
  d[1][1] = -t * ((p3[0] - p2[0]) * (p0[2] - p2[2]) - (p0[0] - p2[0]) * (p3[2] - p2[2]));
  d[1][2] = +t * ((p3[0] - p2[0]) * (p0[1] - p2[1]) - (p0[0] - p2[0]) * (p3[1] - p2[1]));
  d[2][0] = -t * ((p0[1] - p3[1]) * (p1[2] - p3[2]) - (p1[1] - p3[1]) * (p0[2] - p3[2]));
  d[2][1] = +t * ((p0[0] - p3[0]) * (p1[2] - p3[2]) - (p1[0] - p3[0]) * (p0[2] - p3[2]));
  d[2][2] = -t * ((p0[0] - p3[0]) * (p1[1] - p3[1]) - (p1[0] - p3[0]) * (p0[1] - p3[1]));
  d[3][0] = +t * ((p1[1] - p0[1]) * (p2[2] - p0[2]) - (p2[1] - p0[1]) * (p1[2] - p0[2]));
  d[3][1] = -t * ((p1[0] - p0[0]) * (p2[2] - p0[2]) - (p2[0] - p0[0]) * (p1[2] - p0[2]));
  d[3][2] = +t * ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]));
}

static int check_conn(int n, int nelem, int nno, const int* conn) {
  for (long k = 0; k < (long)nelem * nno; ++k)
    if (conn[k] < 0 || conn[k] >= n) return 0;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Element assembly                                                          */
/* ------------------------------------------------------------------------ */

/* femeqn/eqn_poisson.cpp:49-125 (AddLinearSystem_Poisson2D_P1); the per-element
 * coefficient multiplies alpha: alpha_e = alpha*coef[e]. */
int dfo_assemble_poisson2d(int n, const int* rowptr, const int* colind,
                           int nelem, const int* conn, const double* coords,
                           const double* coef, double alpha0, double source,
                           const double* u, double* diag, double* offd, double* res) {
  if (!check_conn(n, nelem, 3, conn)) return -1;
  Merger m; merger_init(&m, n, 1, rowptr, colind, diag, offd);
  for (long e = 0; e < nelem; ++e) {
    const int* no = &conn[e * 3];
    const double alpha = coef ? alpha0 * coef[e] : alpha0;
    double c[3][2], val[3];
    for (int k = 0; k < 3; ++k) {
      c[k][0] = coords[no[k] * 2 + 0]; c[k][1] = coords[no[k] * 2 + 1];
      val[k] = u ? u[no[k]] : 0.0;
    }
    const double area = tri_area(c[0], c[1], c[2]);
    double d[3][2]; tri_dldx(d, c[0], c[1], c[2]);
    double emat[3][3], eres[3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        emat[i][j] = alpha * area * (d[i][0] * d[j][0] + d[i][1] * d[j][1]);
    for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.33333333333333333;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) eres[i] -= emat[i][j] * val[j];
    merge(&m, 3, no, &emat[0][0]);
    for (int i = 0; i < 3; ++i) res[no[i]] += eres[i];
  }
  merger_free(&m);
  return 0;
}

/* femeqn/eqn_poisson.cpp:249-323 (AddLinearSystem_Poisson3D_P1) */
int dfo_assemble_poisson3d(int n, const int* rowptr, const int* colind,
                           int nelem, const int* conn, const double* coords,
                           const double* coef, double alpha0, double source,
                           const double* u, double* diag, double* offd, double* res) {
  if (!check_conn(n, nelem, 4, conn)) return -1;
  Merger m; merger_init(&m, n, 1, rowptr, colind, diag, offd);
  for (long e = 0; e < nelem; ++e) {
    const int* no = &conn[e * 4];
    const double alpha = coef ? alpha0 * coef[e] : alpha0;
    double c[4][3], val[4];
    for (int k = 0; k < 4; ++k) {
      for (int a = 0; a < 3; ++a) c[k][a] = coords[no[k] * 3 + a];
      val[k] = u ? u[no[k]] : 0.0;
    }
    const double vol = tet_volume(c[0], c[1], c[2], c[3]);
    double d[4][3]; tet_dldx(d, c[0], c[1], c[2], c[3]);
    double emat[4][4], eres[4];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        emat[i][j] = alpha * vol * (d[i][0] * d[j][0] + d[i][1] * d[j][1] + d[i][2] * d[j][2]);
    for (int i = 0; i < 4; ++i) eres[i] = source * vol * 0.25;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) eres[i] -= emat[i][j] * val[j];
    merge(&m, 4, no, &emat[0][0]);
    for (int i = 0; i < 4; ++i) res[no[i]] += eres[i];
  }
  merger_free(&m);
  return 0;
}

/* femeqn/eqn_diffusion.cpp:240-347 (AddLinearSystem_Diffusion2D_P1):
 * emat = M + gamma*dt*K, eres = f - K(u + dt*v) - M v; alpha_e = alpha*coef[e]. */
int dfo_assemble_diffusion2d(int n, const int* rowptr, const int* colind,
                             int nelem, const int* conn, const double* coords,
                             const double* coef, double rho, double alpha0, double source,
                             double gamma, double dt, const double* u, const double* v,
                             double* diag, double* offd, double* res) {
  if (!check_conn(n, nelem, 3, conn)) return -1;
  Merger m; merger_init(&m, n, 1, rowptr, colind, diag, offd);
  for (long e = 0; e < nelem; ++e) {
    const int* no = &conn[e * 3];
    const double alpha = coef ? alpha0 * coef[e] : alpha0;
    double c[3][2], val[3], vval[3];
    for (int k = 0; k < 3; ++k) {
      c[k][0] = coords[no[k] * 2 + 0]; c[k][1] = coords[no[k] * 2 + 1];
      val[k] = u ? u[no[k]] : 0.0;
      vval[k] = v ? v[no[k]] : 0.0;
    }
    const double area = tri_area(c[0], c[1], c[2]);
    double d[3][2]; tri_dldx(d, c[0], c[1], c[2]);
    double eC[3][3], eM[3][3], emat[3][3], eres[3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        eC[i][j] = alpha * area * (d[i][0] * d[j][0] + d[i][1] * d[j][1]);
    {
      const double t = rho * area * 0.08333333333333333;
      for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) eM[i][j] = t;
        eM[i][i] += t;
      }
    }
    for (int i = 0; i < 3; ++i) eres[i] = source * area * 0.333333333333333333;
    {
      const double t = gamma * dt;
      for (int k = 0; k < 9; ++k) (&emat[0][0])[k] = (&eM[0][0])[k] + t * (&eC[0][0])[k];
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        eres[i] -= eC[i][j] * (val[j] + dt * vval[j]) + eM[i][j] * vval[j];
    merge(&m, 3, no, &emat[0][0]);
    for (int i = 0; i < 3; ++i) res[no[i]] += eres[i];
  }
  merger_free(&m);
  return 0;
}

/* femeqn/eqn_linear_solid2d.cpp:505-598 (AddLinSys_LinearSolid2D_Static_P1);
 * lambda_e = lambda*coef[e], myu_e = myu*coef[e]. */
int dfo_assemble_solid2d(int n, const int* rowptr, const int* colind,
                         int nelem, const int* conn, const double* coords,
                         const double* coef, double lambda0, double myu0,
                         double rho, double g_x, double g_y,
                         const double* u, double* diag, double* offd, double* res) {
  if (!check_conn(n, nelem, 3, conn)) return -1;
  Merger m; merger_init(&m, n, 2, rowptr, colind, diag, offd);
  for (long e = 0; e < nelem; ++e) {
    const int* no = &conn[e * 3];
    const double lambda = coef ? lambda0 * coef[e] : lambda0;
    const double myu = coef ? myu0 * coef[e] : myu0;
    double c[3][2], disp[3][2];
    for (int k = 0; k < 3; ++k) {
      c[k][0] = coords[no[k] * 2 + 0]; c[k][1] = coords[no[k] * 2 + 1];
      disp[k][0] = u ? u[no[k] * 2 + 0] : 0.0;
      disp[k][1] = u ? u[no[k] * 2 + 1] : 0.0;
    }
    const double area = tri_area(c[0], c[1], c[2]);
    double d[3][2]; tri_dldx(d, c[0], c[1], c[2]);
    double emat[3][3][2][2], eres[3][2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        emat[i][j][0][0] = area * (lambda + myu) * d[i][0] * d[j][0];
        emat[i][j][0][1] = area * (lambda * d[i][0] * d[j][1] + myu * d[j][0] * d[i][1]);
        emat[i][j][1][0] = area * (lambda * d[i][1] * d[j][0] + myu * d[j][1] * d[i][0]);
        emat[i][j][1][1] = area * (lambda + myu) * d[i][1] * d[j][1];
        const double t = (d[i][1] * d[j][1] + d[i][0] * d[j][0]) * area * myu;
        emat[i][j][0][0] += t;
        emat[i][j][1][1] += t;
      }
    for (int i = 0; i < 3; ++i) {
      eres[i][0] = area * rho * g_x * 0.33333333333333333;
      eres[i][1] = area * rho * g_y * 0.33333333333333333;
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        eres[i][0] -= emat[i][j][0][0] * disp[j][0] + emat[i][j][0][1] * disp[j][1];
        eres[i][1] -= emat[i][j][1][0] * disp[j][0] + emat[i][j][1][1] * disp[j][1];
      }
    merge(&m, 3, no, &emat[0][0][0][0]);
    for (int i = 0; i < 3; ++i) {
      res[no[i] * 2 + 0] += eres[i][0];
      res[no[i] * 2 + 1] += eres[i][1];
    }
  }
  merger_free(&m);
  return 0;
}

/* femeqn/eqn_linear_solid3d.cpp:241-334 (AddLinSys_LinearSolid3D_Static_P1) */
int dfo_assemble_solid3d(int n, const int* rowptr, const int* colind,
                         int nelem, const int* conn, const double* coords,
                         const double* coef, double lambda0, double myu0,
                         double rho, double g_x, double g_y, double g_z,
                         const double* u, double* diag, double* offd, double* res) {
  if (!check_conn(n, nelem, 4, conn)) return -1;
  Merger m; merger_init(&m, n, 3, rowptr, colind, diag, offd);
  for (long e = 0; e < nelem; ++e) {
    const int* no = &conn[e * 4];
    const double lambda = coef ? lambda0 * coef[e] : lambda0;
    const double myu = coef ? myu0 * coef[e] : myu0;
    double c[4][3], disp[4][3];
    for (int k = 0; k < 4; ++k)
      for (int a = 0; a < 3; ++a) {
        c[k][a] = coords[no[k] * 3 + a];
        disp[k][a] = u ? u[no[k] * 3 + a] : 0.0;
      }
    const double vol = tet_volume(c[0], c[1], c[2], c[3]);
    double d[4][3]; tet_dldx(d, c[0], c[1], c[2], c[3]);
    double emat[4][4][3][3], eres[4][3];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        for (int a = 0; a < 3; ++a)
          for (int q = 0; q < 3; ++q)
            emat[i][j][a][q] = vol * (lambda * d[i][a] * d[j][q] + myu * d[j][a] * d[i][q]);
        const double t = d[i][0] * d[j][0] + d[i][1] * d[j][1] + d[i][2] * d[j][2];
        emat[i][j][0][0] += vol * myu * t;
        emat[i][j][1][1] += vol * myu * t;
        emat[i][j][2][2] += vol * myu * t;
      }
    for (int i = 0; i < 4; ++i) {
      eres[i][0] = vol * rho * g_x * 0.25;
      eres[i][1] = vol * rho * g_y * 0.25;
      eres[i][2] = vol * rho * g_z * 0.25;
      for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a)
          eres[i][a] -= emat[i][j][a][0] * disp[j][0] + emat[i][j][a][1] * disp[j][1] + emat[i][j][a][2] * disp[j][2];
    }
    merge(&m, 4, no, &emat[0][0][0][0]);
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) res[no[i] * 3 + a] += eres[i][a];
  }
  merger_free(&m);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Dirichlet finalize                                                        */
/* ------------------------------------------------------------------------ */

/* matvec/matdia_blkcrs.cpp:314-343 (fixed block size branch),
 * include/delfem/matvec/bcflag_blk.h:102-129, ls/linearsystem.cpp:92-128 */
double dfo_finalize(int n, int b, const int* rowptr, const int* colind,
                    const int* bcflag, double* diag, double* offd, double* res) {
  const int bs = b * b;
  for (int i = 0; i < n; ++i)
    for (int id = 0; id < b; ++id) {
      if (bcflag[i * b + id] == 0) continue;
      for (int k = 0; k < b; ++k) diag[(long)i * bs + k * b + id] = 0.0;
      for (int j = 0; j < b; ++j) diag[(long)i * bs + id * b + j] = 0.0;
      diag[(long)i * bs + id * b + id] = 1.0;
      for (int c = rowptr[i]; c < rowptr[i + 1]; ++c)
        for (int j = 0; j < b; ++j) offd[(long)c * bs + id * b + j] = 0.0;
    }
  const long nnz = rowptr[n];
  for (long c = 0; c < nnz; ++c) {
    const int jb = colind[c];
    for (int jd = 0; jd < b; ++jd) {
      if (bcflag[jb * b + jd] == 0) continue;
      for (int id = 0; id < b; ++id) offd[c * bs + id * b + jd] = 0.0;
    }
  }
  for (long k = 0; k < (long)n * b; ++k)
    if (bcflag[k] == 1) res[k] = 0;
  double s = 0.0;
  for (long k = 0; k < (long)n * b; ++k) s += res[k] * res[k];
  return sqrt(0.0 + s);
}

/* ------------------------------------------------------------------------ */
/* ILU(0) numeric factorisation -- matvec/matdiafrac_blkcrs.cpp:774-1107      */
/* ------------------------------------------------------------------------ */

/* CalcInvMat (matdiafrac_blkcrs.cpp:107-136): in-place Gauss-Jordan, info=1
 * on a pivot below 1e-30 (left partially processed, as in the reference). */
static void inv_gauss_jordan(double* a, int n, int* info) {
  *info = 0;
  for (int i = 0; i < n; ++i) {
    if (fabs(a[i * n + i]) < 1.0e-30) { *info = 1; return; }
    if (a[i * n + i] < 0.0) (*info)--;
    double t = 1.0 / a[i * n + i];
    a[i * n + i] = 1.0;
    for (int k = 0; k < n; ++k) a[i * n + k] *= t;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      t = a[j * n + i];
      a[j * n + i] = 0.0;
      for (int k = 0; k < n; ++k) a[j * n + k] -= t * a[i * n + k];
    }
  }
}

int dfo_ilu0(int n, int b, const int* rowptr, const int* colind, const int* diaind,
             double* diag, double* offd) {
  const int bs = b * b;
  const int nmax_sing = 10;
  int icnt_sing = 0;
  int* row2crs = (int*)malloc(sizeof(int) * ((size_t)n + 1));
  for (int j = 0; j < n; ++j) row2crs[j] = -1;
  double tmp[81];
  for (int i = 0; i < n; ++i) {
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) row2crs[colind[c]] = c;
    /* A_ij -= A_ik * U'_kj for k in L(i), j in U(k) */
    for (int ik = rowptr[i]; ik < diaind[i]; ++ik) {
      const int k = colind[ik];
      const double* pik = &offd[(long)ik * bs];
      for (int kj = diaind[k]; kj < rowptr[k + 1]; ++kj) {
        const int j = colind[kj];
        const double* pkj = &offd[(long)kj * bs];
        double* pij;
        if (j != i) {
          const int ij = row2crs[j];
          if (ij == -1) continue;
          pij = &offd[(long)ij * bs];
        } else {
          pij = &diag[(long)i * bs];
        }
        if (b == 1) {
          pij[0] -= pik[0] * pkj[0];
        } else if (b == 2) {
          pij[0] -= pik[0] * pkj[0] + pik[1] * pkj[2];
          pij[1] -= pik[0] * pkj[1] + pik[1] * pkj[3];
          pij[2] -= pik[2] * pkj[0] + pik[3] * pkj[2];
          pij[3] -= pik[2] * pkj[1] + pik[3] * pkj[3];
        } else if (b == 3) {
          for (int r = 0; r < 3; ++r) {
            pij[r * 3 + 0] -= pik[r * 3 + 0] * pkj[0] + pik[r * 3 + 1] * pkj[3] + pik[r * 3 + 2] * pkj[6];
            pij[r * 3 + 1] -= pik[r * 3 + 0] * pkj[1] + pik[r * 3 + 1] * pkj[4] + pik[r * 3 + 2] * pkj[7];
            pij[r * 3 + 2] -= pik[r * 3 + 0] * pkj[2] + pik[r * 3 + 1] * pkj[5] + pik[r * 3 + 2] * pkj[8];
          }
        } else {
          /* CalcSubMatPr (matdiafrac_blkcrs.cpp:62-73): one subtraction per term */
          for (int r = 0; r < b; ++r)
            for (int q = 0; q < b; ++q)
              for (int t = 0; t < b; ++t) pij[r * b + q] -= pik[r * b + t] * pkj[t * b + q];
        }
      }
    }
    /* invert the pivot block */
    double* pii = &diag[(long)i * bs];
    int sing = 0;
    if (b == 1) {
      const double v = pii[0];
      if (fabs(v) > 1.0e-30) pii[0] = 1.0 / v; else sing = 1;
    } else if (b == 2) {
      const double det = pii[0] * pii[3] - pii[1] * pii[2];
      if (fabs(det) > 1.0e-30) {
        const double inv_det = 1.0 / det;
        const double t = pii[0];
        pii[0] = inv_det * pii[3];
        pii[1] = -inv_det * pii[1];
        pii[2] = -inv_det * pii[2];
        pii[3] = inv_det * t;
      } else sing = 1;
    } else if (b == 3) {
      const double* a = pii;
      const double det = a[0] * a[4] * a[8] + a[3] * a[7] * a[2] + a[6] * a[1] * a[5]
                       - a[0] * a[7] * a[5] - a[6] * a[4] * a[2] - a[3] * a[1] * a[8];
      if (fabs(det) > 1.0e-30) {
        /* CalcInvMat3 (matdiafrac_blkcrs.cpp:139-158) recomputes det identically */
        const double inv_det = 1.0 / det;
        for (int k = 0; k < 9; ++k) tmp[k] = pii[k];
        const double* t = tmp;
        pii[0] = inv_det * (t[4] * t[8] - t[5] * t[7]);
        pii[1] = inv_det * (t[2] * t[7] - t[1] * t[8]);
        pii[2] = inv_det * (t[1] * t[5] - t[2] * t[4]);
        pii[3] = inv_det * (t[5] * t[6] - t[3] * t[8]);
        pii[4] = inv_det * (t[0] * t[8] - t[2] * t[6]);
        pii[5] = inv_det * (t[2] * t[3] - t[0] * t[5]);
        pii[6] = inv_det * (t[3] * t[7] - t[4] * t[6]);
        pii[7] = inv_det * (t[1] * t[6] - t[0] * t[7]);
        pii[8] = inv_det * (t[0] * t[4] - t[1] * t[3]);
      } else sing = 1;
    } else {
      int info = 0;
      inv_gauss_jordan(pii, b, &info);
      if (info == 1) sing = 1;
    }
    if (sing) {
      icnt_sing++;
      if (icnt_sing > nmax_sing) { free(row2crs); return -1; }
    }
    /* U'_ij = D_i^-1 * A_ij for j > i */
    for (int ij = diaind[i]; ij < rowptr[i + 1]; ++ij) {
      double* pij = &offd[(long)ij * bs];
      if (b == 1) {
        pij[0] = pij[0] * pii[0];
      } else if (b == 2) {
        for (int k = 0; k < 4; ++k) tmp[k] = pij[k];
        pij[0] = pii[0] * tmp[0] + pii[1] * tmp[2];
        pij[1] = pii[0] * tmp[1] + pii[1] * tmp[3];
        pij[2] = pii[2] * tmp[0] + pii[3] * tmp[2];
        pij[3] = pii[2] * tmp[1] + pii[3] * tmp[3];
      } else if (b == 3) {
        for (int k = 0; k < 9; ++k) tmp[k] = pij[k];
        for (int r = 0; r < 3; ++r) {
          pij[r * 3 + 0] = pii[r * 3 + 0] * tmp[0] + pii[r * 3 + 1] * tmp[3] + pii[r * 3 + 2] * tmp[6];
          pij[r * 3 + 1] = pii[r * 3 + 0] * tmp[1] + pii[r * 3 + 1] * tmp[4] + pii[r * 3 + 2] * tmp[7];
          pij[r * 3 + 2] = pii[r * 3 + 0] * tmp[2] + pii[r * 3 + 1] * tmp[5] + pii[r * 3 + 2] * tmp[8];
        }
      } else {
        /* CalcMatPr (matdiafrac_blkcrs.cpp:45-60): A_ij = A_ii * A_ij */
        for (int k = 0; k < bs; ++k) tmp[k] = pij[k];
        for (int r = 0; r < b; ++r)
          for (int q = 0; q < b; ++q) {
            double s = 0.0;
            for (int t = 0; t < b; ++t) s += pii[r * b + t] * tmp[t * b + q];
            pij[r * b + q] = s;
          }
      }
    }
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) row2crs[colind[c]] = -1;
  }
  free(row2crs);
  return icnt_sing;
}

/* ------------------------------------------------------------------------ */
/* Triangular sweeps -- matvec/matdiafrac_blkcrs.cpp:332-669                 */
/* ------------------------------------------------------------------------ */

void dfo_forward(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                 const double* fdiag, const double* foffd, double* vec) {
  const int bs = b * b;
  double t[9];
  for (int i = 0; i < n; ++i) {
    double* vi = &vec[(long)i * b];
    for (int d = 0; d < b; ++d) t[d] = vi[d];
    for (int c = rowptr[i]; c < diaind[i]; ++c) {
      const double* L = &foffd[(long)c * bs];
      const double* vj = &vec[(long)colind[c] * b];
      if (b == 1) {
        t[0] -= L[0] * vj[0];
      } else if (b == 2) {
        const double v0 = vj[0], v1 = vj[1];
        t[0] -= L[0] * v0 + L[1] * v1;
        t[1] -= L[2] * v0 + L[3] * v1;
      } else if (b == 3) {
        const double v0 = vj[0], v1 = vj[1], v2 = vj[2];
        t[0] -= L[0] * v0 + L[1] * v1 + L[2] * v2;
        t[1] -= L[3] * v0 + L[4] * v1 + L[5] * v2;
        t[2] -= L[6] * v0 + L[7] * v1 + L[8] * v2;
      } else {
        for (int r = 0; r < b; ++r)
          for (int q = 0; q < b; ++q) t[r] -= L[r * b + q] * vj[q];
      }
    }
    const double* D = &fdiag[(long)i * bs];
    if (b == 1) {
      vi[0] = D[0] * t[0];
    } else if (b == 2) {
      vi[0] = D[0] * t[0] + D[1] * t[1];
      vi[1] = D[2] * t[0] + D[3] * t[1];
    } else if (b == 3) {
      vi[0] = D[0] * t[0] + D[1] * t[1] + D[2] * t[2];
      vi[1] = D[3] * t[0] + D[4] * t[1] + D[5] * t[2];
      vi[2] = D[6] * t[0] + D[7] * t[1] + D[8] * t[2];
    } else {
      for (int r = 0; r < b; ++r) {
        double s = 0.0;
        for (int q = 0; q < b; ++q) s += D[r * b + q] * t[q];
        vi[r] = s;
      }
    }
  }
}

void dfo_backward(int n, int b, const int* rowptr, const int* colind, const int* diaind,
                  const double* foffd, double* vec) {
  const int bs = b * b;
  double t[9];
  for (int i = n - 1; i >= 0; --i) {
    double* vi = &vec[(long)i * b];
    for (int d = 0; d < b; ++d) t[d] = vi[d];
    for (int c = diaind[i]; c < rowptr[i + 1]; ++c) {
      const double* U = &foffd[(long)c * bs];
      const double* vj = &vec[(long)colind[c] * b];
      if (b == 1) {
        t[0] -= U[0] * vj[0];
      } else if (b == 2) {
        const double v0 = vj[0], v1 = vj[1];
        t[0] -= U[0] * v0 + U[1] * v1;
        t[1] -= U[2] * v0 + U[3] * v1;
      } else if (b == 3) {
        const double v0 = vj[0], v1 = vj[1], v2 = vj[2];
        t[0] -= U[0] * v0 + U[1] * v1 + U[2] * v2;
        t[1] -= U[3] * v0 + U[4] * v1 + U[5] * v2;
        t[2] -= U[6] * v0 + U[7] * v1 + U[8] * v2;
      } else {
        for (int r = 0; r < b; ++r)
          for (int q = 0; q < b; ++q) t[r] -= U[r * b + q] * vj[q];
      }
    }
    for (int d = 0; d < b; ++d) vi[d] = t[d];
  }
}

/* ------------------------------------------------------------------------ */
/* SpMV -- matvec/matdia_blkcrs.cpp:966-1094                                 */
/* ------------------------------------------------------------------------ */

void dfo_matvec(int n, int b, const int* rowptr, const int* colind,
                const double* diag, const double* offd,
                double alpha, const double* x, double beta, double* y) {
  const int bs = b * b;
  for (int i = 0; i < n; ++i) {
    double* yi = &y[(long)i * b];
    for (int d = 0; d < b; ++d) yi[d] *= beta;
    for (int c = rowptr[i]; c < rowptr[i + 1]; ++c) {
      const double* A = &offd[(long)c * bs];
      const double* xj = &x[(long)colind[c] * b];
      if (b == 1) {
        yi[0] += alpha * A[0] * xj[0];
      } else if (b == 2) {
        yi[0] += alpha * (A[0] * xj[0] + A[1] * xj[1]);
        yi[1] += alpha * (A[2] * xj[0] + A[3] * xj[1]);
      } else if (b == 3) {
        yi[0] += alpha * (A[0] * xj[0] + A[1] * xj[1] + A[2] * xj[2]);
        yi[1] += alpha * (A[3] * xj[0] + A[4] * xj[1] + A[5] * xj[2]);
        yi[2] += alpha * (A[6] * xj[0] + A[7] * xj[1] + A[8] * xj[2]);
      } else {
        for (int r = 0; r < b; ++r)
          for (int q = 0; q < b; ++q) yi[r] += alpha * A[r * b + q] * xj[q];
      }
    }
    const double* D = &diag[(long)i * bs];
    const double* xi = &x[(long)i * b];
    if (b == 1) {
      yi[0] += alpha * D[0] * xi[0];
    } else if (b == 2) {
      yi[0] += alpha * (D[0] * xi[0] + D[1] * xi[1]);
      yi[1] += alpha * (D[2] * xi[0] + D[3] * xi[1]);
    } else if (b == 3) {
      yi[0] += alpha * (D[0] * xi[0] + D[1] * xi[1] + D[2] * xi[2]);
      yi[1] += alpha * (D[3] * xi[0] + D[4] * xi[1] + D[5] * xi[2]);
      yi[2] += alpha * (D[6] * xi[0] + D[7] * xi[1] + D[8] * xi[2]);
    } else {
      for (int r = 0; r < b; ++r)
        for (int q = 0; q < b; ++q) yi[r] += alpha * D[r * b + q] * xi[q];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* PCG -- ls/solver_ls_iter.cpp:100-172 over ls/linearsystem.cpp:250-415     */
/* ------------------------------------------------------------------------ */

static double vdot(long m, const double* a, const double* b) {
  double s = 0.0;
  for (long k = 0; k < m; ++k) s += a[k] * b[k];
  return 0.0 + s; /* CLinearSystem::DOT accumulates the segment dot into 0.0 */
}
static void vaxpy(long m, double alpha, const double* x, double* y) {
  if (alpha == 0) return; /* CLinearSystem::AXPY returns early on alpha == 0 */
  for (long k = 0; k < m; ++k) y[k] += alpha * x[k];
}
static void vscal(long m, double alpha, double* x) {
  for (long k = 0; k < m; ++k) x[k] *= alpha;
}

int dfo_pcg(int n, int b, const int* rowptr, const int* colind, const int* diaind,
            const double* diag, const double* offd,
            const double* fdiag, const double* foffd,
            double* r, double* x, double* conv, unsigned* iter, double* work) {
  return dfo_pcg_f(n, b, rowptr, colind, diag, offd, rowptr, colind, diaind, fdiag, foffd, r, x, conv, iter,
                   work);
}

int dfo_pcg_f(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
              const int* rowptr_f, const int* colind_f, const int* diaind_f,
              const double* fdiag, const double* foffd,
              double* r, double* x, double* conv, unsigned* iter, double* work) {
  const long m = (long)n * b;
  const double tol = *conv;
  const unsigned mx_iter = *iter;
  double* p = work;
  double* z = work + m;
  vscal(m, 0.0, x);
  double sq_inv_norm_res0;
  {
    const double s0 = vdot(m, r, r);
    if (s0 < 1.0e-30) { *conv = 0.0; *iter = 0; return 1; }
    sq_inv_norm_res0 = 1.0 / s0;
  }
  memcpy(z, r, sizeof(double) * (size_t)m);
  dfo_forward(n, b, rowptr_f, colind_f, diaind_f, fdiag, foffd, z);
  dfo_backward(n, b, rowptr_f, colind_f, diaind_f, foffd, z);
  memcpy(p, z, sizeof(double) * (size_t)m);
  double rz = vdot(m, r, z);
  for (unsigned it = 0; it < mx_iter; ++it) {
    dfo_matvec(n, b, rowptr, colind, diag, offd, 1.0, p, 0.0, z);
    const double pAp = vdot(m, p, z);
    const double alpha = rz / pAp;
    vaxpy(m, -alpha, z, r);
    vaxpy(m, alpha, p, x);
    {
      const double sq = vdot(m, r, r);
      if (sq * sq_inv_norm_res0 < tol * tol) {
        *conv = sqrt(sq * sq_inv_norm_res0);
        *iter = it;
        return 1;
      }
    }
    memcpy(z, r, sizeof(double) * (size_t)m);
    dfo_forward(n, b, rowptr_f, colind_f, diaind_f, fdiag, foffd, z);
    dfo_backward(n, b, rowptr_f, colind_f, diaind_f, foffd, z);
    const double rz_new = vdot(m, r, z);
    const double beta = rz_new / rz;
    rz = rz_new;
    vscal(m, beta, p);
    vaxpy(m, 1.0, z, p);
  }
  {
    const double sq = vdot(m, r, r);
    *conv = sqrt(sq * sq_inv_norm_res0);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Preconditioned BiCGSTAB -- LsSol::Solve_PBiCGSTAB                          */
/* (ls/solver_ls_iter.cpp:291-408), one COPY / DOT / AXPY / SCAL / MATVEC /   */
/* SolvePrecond per call of the reference, in its order                       */
/* ------------------------------------------------------------------------ */

int dfo_bicgstab(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                 const int* rowptr_f, const int* colind_f, const int* diaind_f,
                 const double* fdiag, const double* foffd,
                 double* r, double* x, double* conv, unsigned* iter, double* work) {
  return dfo_bicgstab_hist(n, b, rowptr, colind, diag, offd, rowptr_f, colind_f, diaind_f, fdiag, foffd, r, x, conv,
                           iter, work, NULL);
}

int dfo_bicgstab_hist(int n, int b, const int* rowptr, const int* colind, const double* diag, const double* offd,
                      const int* rowptr_f, const int* colind_f, const int* diaind_f,
                      const double* fdiag, const double* foffd,
                      double* r, double* x, double* conv, unsigned* iter, double* work, double* hist) {
  const long m = (long)n * b;
  const size_t vb = sizeof(double) * (size_t)m;
  const double tol = *conv;
  const unsigned mx_iter = *iter;
  double* s = work;
  double* ms = work + m;
  double* ams = work + 2 * m;
  double* p = work + 3 * m;
  double* mp = work + 4 * m;
  double* amp = work + 5 * m;
  double* r2 = work + 6 * m;
  double sq_inv_norm_res_ini;
  {
    const double sq = vdot(m, r, r);
    if (sq < 1.0e-60) { /* x is left as it is */
      *conv = sqrt(sq);
      *iter = 0;
      return 1;
    }
    sq_inv_norm_res_ini = 1.0 / sq;
  }
  vscal(m, 0.0, x);
  memcpy(r2, r, vb);
  memcpy(p, r, vb);
  *iter = mx_iter;
  for (unsigned it = 1; it < mx_iter; ++it) {
    memcpy(mp, p, vb);
    dfo_forward(n, b, rowptr_f, colind_f, diaind_f, fdiag, foffd, mp);
    dfo_backward(n, b, rowptr_f, colind_f, diaind_f, foffd, mp);
    const double r_r2 = vdot(m, r, r2);
    dfo_matvec(n, b, rowptr, colind, diag, offd, 1.0, mp, 0.0, amp);
    const double alpha = r_r2 / vdot(m, amp, r2);
    memcpy(s, r, vb);
    vaxpy(m, -alpha, amp, s);
    memcpy(ms, s, vb);
    dfo_forward(n, b, rowptr_f, colind_f, diaind_f, fdiag, foffd, ms);
    dfo_backward(n, b, rowptr_f, colind_f, diaind_f, foffd, ms);
    dfo_matvec(n, b, rowptr, colind, diag, offd, 1.0, ms, 0.0, ams);
    double omega;
    {
      const double den = vdot(m, ams, ams);
      const double num = vdot(m, s, ams);
      omega = num / den;
    }
    vaxpy(m, alpha, mp, x);
    vaxpy(m, omega, ms, x);
    memcpy(r, s, vb);
    vaxpy(m, -omega, ams, r);
    {
      const double sq = vdot(m, r, r);
      if (hist) hist[it] = sq * sq_inv_norm_res_ini;
      if (sq * sq_inv_norm_res_ini < tol * tol) {
        *conv = sqrt(sq * sq_inv_norm_res_ini);
        *iter = it;
        return 1;
      }
    }
    const double beta = vdot(m, r, r2) * alpha / (r_r2 * omega);
    vscal(m, beta, p);
    vaxpy(m, 1.0, r, p);
    vaxpy(m, -beta * omega, amp, p);
  }
  return 0; /* the reference returns true here too, with *conv untouched */
}
