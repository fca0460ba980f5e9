/*
 * sbm_oracle.c -- CPU oracle for the SBM hot path (test infrastructure).
 *
 * A line-by-line FP64 restatement of the reference Fortran, used only as the
 * checker (tests/, __graft_entry__.smoke(), bench.py's CPU baseline leg).
 * Pinned against the reference's own Fortran, run by an interpreter
 * (tests/golden/reference_v1.npz); see sbm_oracle.h for the rules this file
 * keeps.
 *
 * File references are to AffanMalik90/Elsim:
 *   SBMES = src/frtrn/SBMES_3D_MPI_CH_Gr_CONJG_VD_T05_01_BQ_hx3.f90
 *   LS    = src/frtrn/LevelSet_3D.f90
 *   AD    = src/frtrn/AccDiff_3D.f90
 *   RM    = src/frtrn/RM_UCNCT_3D.f90
 */
#include "sbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX(i, j, k) ((size_t)(i) + (size_t)(ny + 2) * ((size_t)(j) + (size_t)(nx + 2) * (size_t)(k)))
#define NH ((size_t)(ny + 2) * (size_t)(nx + 2) * (size_t)(nz + 2))

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the following parallel regions of the calling host thread
 * (the CPU baseline times one thread and all of them); n <= 0 restores the
 * count the library started with.  Results do not depend on it. */
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  static int initial = 0;
  if (!initial) initial = omp_get_max_threads();
  omp_set_num_threads(n > 0 ? n : initial);
#else
  (void)n;
#endif
}

/* --------------------------------------------------------------- ghosts */

/* NoGrdBc3D, LS:164-190 (same as RM:180-205). */
void orc_nogrdbc(int py, int px, int pz, double* f) {
  const int ny = py, nx = px, nz = pz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j) {
      f[IX(0, j, k)] = f[IX(1, j, k)];
      f[IX(ny + 1, j, k)] = f[IX(ny, j, k)];
    }
  for (int k = 1; k <= nz; ++k)
    for (int i = 0; i <= ny + 1; ++i) {
      f[IX(i, 0, k)] = f[IX(i, 1, k)];
      f[IX(i, nx + 1, k)] = f[IX(i, nx, k)];
    }
  for (int j = 0; j <= nx + 1; ++j)
    for (int i = 0; i <= ny + 1; ++i) {
      f[IX(i, j, 0)] = f[IX(i, j, 1)];
      f[IX(i, j, nz + 1)] = f[IX(i, j, nz)];
    }
}

/* BcMpiYZ on a single rank (rnb = cnb = 1), SBMES:1043-1088: the z halo
 * of the interior columns, then the y halo over 0:nz+1, both edge copies. */
void orc_bc_yz(int ny, int nx, int nz, double* f) {
  for (int j = 1; j <= nx; ++j)
    for (int i = 1; i <= ny; ++i) f[IX(i, j, 0)] = f[IX(i, j, 1)];
  for (int j = 1; j <= nx; ++j)
    for (int i = 1; i <= ny; ++i) f[IX(i, j, nz + 1)] = f[IX(i, j, nz)];
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 1; j <= nx; ++j) f[IX(0, j, k)] = f[IX(1, j, k)];
  for (int k = 0; k <= nz + 1; ++k)
    for (int j = 1; j <= nx; ++j) f[IX(ny + 1, j, k)] = f[IX(ny, j, k)];
}

/* The x-face lines written after each BcMpiYZ call, e.g. SBMES:437-438,
 * :512-513, :647, :667-668, :718-719: mode 0 copies the edge plane, mode 1
 * writes the value, over rows 0:ny+1 and planes k0:k1. */
void orc_bc_x(int ny, int nx, int nz, double* f, int k0, int k1,
              int mode0, double v0, int mode1, double v1) {
  (void)nz;
  for (int k = k0; k <= k1; ++k)
    for (int i = 0; i <= ny + 1; ++i) {
      f[IX(i, nx + 1, k)] = mode1 ? v1 : f[IX(i, nx, k)];
      f[IX(i, 0, k)] = mode0 ? v0 : f[IX(i, 1, k)];
    }
}

/* ------------------------------------------------------------ reductions */

/* sum over the interior of a(i)*b(i) (b may be NULL), plane by plane. */
static double sum_prod(int ny, int nx, int nz, const double* a, const double* b) {
  double* part = (double*)malloc(sizeof(double) * (size_t)nz);
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k) {
    double s = 0.0;
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        s += b ? a[c] * b[c] : a[c];
      }
    part[k - 1] = s;
  }
  double t = 0.0;
  for (int k = 0; k < nz; ++k) t += part[k];
  free(part);
  return t;
}

/* sum over the interior of a(i)^2 * w(i) (w may be NULL). */
static double sum_sq_w(int ny, int nx, int nz, const double* a, const double* w) {
  double* part = (double*)malloc(sizeof(double) * (size_t)nz);
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k) {
    double s = 0.0;
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double a2 = a[c] * a[c];
        s += w ? a2 * w[c] : a2;
      }
    part[k - 1] = s;
  }
  double t = 0.0;
  for (int k = 0; k < nz; ++k) t += part[k];
  free(part);
  return t;
}

/* sum over the interior of (a-b)^2 * w. */
static double sum_dsq_w(int ny, int nx, int nz, const double* a, const double* b,
                        const double* w) {
  double* part = (double*)malloc(sizeof(double) * (size_t)nz);
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k) {
    double s = 0.0;
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double d = a[c] - b[c];
        s += (d * d) * w[c];
      }
    part[k - 1] = s;
  }
  double t = 0.0;
  for (int k = 0; k < nz; ++k) t += part[k];
  free(part);
  return t;
}

/* Global interior sum of a*b: the reference's local sum + MPI_ALLGATHER +
 * SUM over ranks (e.g. the CG norms of SBMES:524-540), on one domain. */
double orc_dot(int ny, int nx, int nz, const double* a, const double* b) {
  return sum_prod(ny, nx, nz, a, b);
}

/* ------------------------------------------------------------ level set */

/* AbsGrd3DUW_XYZ, LS:265-322: Godunov upwind |grad f| on the interior. */
void orc_absgrd(int py, int px, int pz, const double* sg, const double* f, double* gr) {
  const int ny = py, nx = px, nz = pz;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double ag = f[c] - f[IX(i - 1, j, k)];
        const double bg = f[IX(i + 1, j, k)] - f[c];
        const double cg = f[c] - f[IX(i, j - 1, k)];
        const double dg = f[IX(i, j + 1, k)] - f[c];
        const double eg = f[c] - f[IX(i, j, k - 1)];
        const double fg = f[IX(i, j, k + 1)] - f[c];
        const double s = sg[c];
        if (s == 0.0) {
          gr[c] = 0.0;
        } else if (s > 0.0) {
          double a = ag > 0.0 ? ag : 0.0, b = -bg > 0.0 ? -bg : 0.0;
          double cc = cg > 0.0 ? cg : 0.0, d = -dg > 0.0 ? -dg : 0.0;
          double e = eg > 0.0 ? eg : 0.0, ff = -fg > 0.0 ? -fg : 0.0;
          double t1 = a * a, t2 = b * b, t3 = cc * cc, t4 = d * d, t5 = e * e, t6 = ff * ff;
          double m1 = t1 > t2 ? t1 : t2, m2 = t3 > t4 ? t3 : t4, m3 = t5 > t6 ? t5 : t6;
          gr[c] = sqrt((m1 + m2) + m3);
        } else if (s < 0.0) {
          double a = -ag > 0.0 ? -ag : 0.0, b = bg > 0.0 ? bg : 0.0;
          double cc = -cg > 0.0 ? -cg : 0.0, d = dg > 0.0 ? dg : 0.0;
          double e = -eg > 0.0 ? -eg : 0.0, ff = fg > 0.0 ? fg : 0.0;
          double t1 = a * a, t2 = b * b, t3 = cc * cc, t4 = d * d, t5 = e * e, t6 = ff * ff;
          double m1 = t1 > t2 ? t1 : t2, m2 = t3 > t4 ? t3 : t4, m3 = t5 > t6 ? t5 : t6;
          gr[c] = sqrt((m1 + m2) + m3);
        }
      }
}

/* Allen-Cahn pre-smoothing of the stacked voxel field, LS:116-136:
 * NoGrdBc3D, then `iters` times
 *   sgF = 2*dsF*(1.0-dsF)*(1.0-2*dsF) - 0.64*(six neighbours - 6*dsF)
 *   dsF = dsF - 0.05*sgF                       (interior, array semantics)
 *   NoGrdBc3D
 * with the REAL(4) literals 0.64 and 0.05 promoted to REAL(8) and the
 * Fortran left-to-right evaluation order. */
void orc_allen_cahn(int iters, int py, int px, int pz, double* f) {
  const int ny = py, nx = px, nz = pz;
  const size_t n = (size_t)(ny + 2) * (nx + 2) * (nz + 2);
  const double c064 = (double)0.64f, c005 = (double)0.05f;
  double* s = (double*)malloc(n * sizeof(double));
  if (!s) return;
  orc_nogrdbc(py, px, pz, f);
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const double d = f[IX(i, j, k)];
          const double lap = f[IX(i + 1, j, k)] + f[IX(i - 1, j, k)] + f[IX(i, j + 1, k)] +
                             f[IX(i, j - 1, k)] + f[IX(i, j, k + 1)] + f[IX(i, j, k - 1)] -
                             6 * d;
          s[IX(i, j, k)] = 2 * d * (1.0 - d) * (1.0 - 2 * d) - c064 * lap;
        }
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) f[IX(i, j, k)] = f[IX(i, j, k)] - c005 * s[IX(i, j, k)];
    orc_nogrdbc(py, px, pz, f);
  }
  free(s);
}

/* The stacked voxel field, LS:80-122, literally: TmpB(yo,zo,xo) from the
 * reorientation loop (:82-84), the tunnel loop over k = 1..zg, j = 1..xg,
 * i = 1..yg writing TmpB(i,j,k) through its column-major address
 * (i-1) + yo*((j-1) + zo*(k-1)) even where j exceeds zo (:87-106), the
 * stacking of nthick thicknesses after xoff zero columns (:109-119: the
 * reference's 4 = straight, mirrored, copy of the first, copy of the second),
 * then NoGrdBc3D (:122).  ds is the halo-padded (yg+2)(xg+2)(zg+2) array,
 * xg = xoff + nthick*zo.  Returns 0, or -1 when an argument is out of range
 * or the tunnel loop would leave TmpB. */
int orc_ls_geometry(const double* vox, int yo, int xo, int zo, int yg, int zg, int xoff,
                    int nthick, double tr, double* ds) {
  const long xg = xoff + (long)nthick * zo;
  if (yo < 1 || xo < 1 || zo < 1 || yg < 1 || zg < 1 || xoff < 0 || nthick < 1 || yg > yo ||
      zg > xo || (xg - 1) + (long)zo * (zg - 1) >= (long)zo * xo)
    return -1;
  const size_t nb = (size_t)yo * zo * xo;
  double* tb = (double*)malloc(nb * sizeof(double));
  if (!tb) return -1;
  /* TmpB(1:yo,k,1:xo) = TmpA(1:yo,1:xo,zo-k+1) */
  for (long k = 1; k <= zo; ++k)
    for (long j = 1; j <= xo; ++j)
      for (long i = 1; i <= yo; ++i)
        tb[(i - 1) + yo * ((k - 1) + zo * (j - 1))] = vox[(i - 1) + yo * ((j - 1) + xo * (zo - k))];
  for (long k = 1; k <= zg; ++k)
    for (long j = 1; j <= xg; ++j)
      for (long i = 1; i <= yg; ++i) {
        const size_t at = (size_t)((i - 1) + yo * ((j - 1) + zo * (k - 1)));
        double rad = sqrt(((double)i - 1.0) * ((double)i - 1.0) +
                          ((double)k - (double)zg) * ((double)k - (double)zg));
        if (rad < tr) tb[at] = 0.0;
        rad = sqrt(((double)i - (double)yg) * ((double)i - (double)yg) +
                   ((double)k - 1.0) * ((double)k - 1.0));
        if (rad < tr) tb[at] = 0.0;
      }
  const int ny = yg, nx = (int)xg, nz = zg;
  for (long k = 1; k <= zg; ++k)
    for (long j = 1; j <= xg; ++j)
      for (long i = 1; i <= yg; ++i) {
        double v = 0.0;
        if (j > xoff) {
          const long t = (j - xoff - 1) / zo, r = (j - xoff - 1) % zo;
          /* thickness 1: TmpB(:,1:zo,:); thickness 2: TmpB(:, j-((j-221)*2+51), :)
           * = column zo..1; later ones repeat the first two */
          const long c = (t % 2 == 0) ? r + 1 : zo - r;
          v = tb[(i - 1) + yo * ((c - 1) + zo * (k - 1))];
        }
        ds[IX(i, j, k)] = v;
      }
  free(tb);
  orc_nogrdbc(yg, (int)xg, zg, ds);
  return 0;
}

/* ReDist3D_XYZ, LS:194-261 (dt = 1.0d-1) and RM:209-276 (dt = 1.0e-1
 * REAL(4)): f_t = sg (1 - |grad f|) on every cell including the ghosts,
 * with the sign-change guard of LS:245-249. */
void orc_redist(int lit, double dt, int py, int px, int pz, const double* sg, double* f) {
  const int ny = py, nx = px, nz = pz;
  const size_t n = NH;
  double* gf = (double*)calloc(n, sizeof(double));
  double* nf = (double*)malloc(n * sizeof(double));
  const double small = dt * 1.0e-7;
  for (int m = 1; m <= lit; ++m) {
    orc_absgrd(py, px, pz, sg, f, gf);
    orc_nogrdbc(py, px, pz, gf);
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)n; ++c) {
      double v = f[c] + (sg[c] * (1.0 - gf[c])) * dt;
      if (!(v * f[c] > 0.0)) v = f[c] + small * sg[c];
      nf[c] = v;
    }
    memcpy(f, nf, n * sizeof(double));
  }
  free(gf);
  free(nf);
}

/* One phase of AccDiff_3D (AD:111-169 solid, AD:185-243 electrolyte) for
 * iterations 2..term.  dirichlet_x = 1: Cn = 1 on x = px+1 and Neumann at
 * x = 0 (solid); 0: Cn = 1 on x = 0 and Neumann at x = px+1. */
void orc_accdiff(int py, int px, int pz, const double* psi, double* cn,
                 int term, int dirichlet_x) {
  const int ny = py, nx = px, nz = pz;
  const double dt = (double)(1.25e-1f * 0.5f); /* AD:51, REAL(4) product */
  const double idh2 = 1.0 / (1.0 * 1.0);        /* AD:49, dh = 1.0e0 */
  const double thr = (double)4.0e-1f;           /* AD:118, :133 */
  const double cmin = (double)1.0e-4f;          /* AD:133 */
  const double cnbv = 1.0;                       /* AD:61 */
  double* div = (double*)calloc(NH, sizeof(double));
  for (int iter = 2; iter <= term; ++iter) {
    /* WHERE (psi >= 0.4): Div from the old Cn everywhere, then Cn update */
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const size_t c = IX(i, j, k);
          const double p = psi[c];
          if (p >= thr) {
            const double u = cn[c];
            double s = (psi[IX(i + 1, j, k)] + p) * (cn[IX(i + 1, j, k)] - u);
            s = s - (p + psi[IX(i - 1, j, k)]) * (u - cn[IX(i - 1, j, k)]);
            s = s + (psi[IX(i, j + 1, k)] + p) * (cn[IX(i, j + 1, k)] - u);
            s = s - (p + psi[IX(i, j - 1, k)]) * (u - cn[IX(i, j - 1, k)]);
            s = s + (psi[IX(i, j, k + 1)] + p) * (cn[IX(i, j, k + 1)] - u);
            s = s - (p + psi[IX(i, j, k - 1)]) * (u - cn[IX(i, j, k - 1)]);
            div[c] = ((0.5 * idh2) / p) * s;
          }
        }
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const size_t c = IX(i, j, k);
          if (psi[c] >= thr) cn[c] = cn[c] + dt * div[c];
        }
    if (iter % 5 == 1) { /* AD:132-134 */
#pragma omp parallel for schedule(static)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= nx; ++j)
          for (int i = 1; i <= ny; ++i) {
            const size_t c = IX(i, j, k);
            if (cn[c] > cmin && psi[c] > thr) cn[c] = 1.0;
          }
    }
    /* AD:138-148 (solid) / AD:212-222 (electrolyte) */
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j) {
        cn[IX(0, j, k)] = cn[IX(1, j, k)];
        cn[IX(ny + 1, j, k)] = cn[IX(ny, j, k)];
      }
    for (int k = 1; k <= nz; ++k)
      for (int i = 0; i <= ny + 1; ++i) {
        if (dirichlet_x) {
          cn[IX(i, 0, k)] = cn[IX(i, 1, k)];
          cn[IX(i, nx + 1, k)] = cnbv;
        } else {
          cn[IX(i, 0, k)] = cnbv;
          cn[IX(i, nx + 1, k)] = cn[IX(i, nx, k)];
        }
      }
    for (int j = 0; j <= nx + 1; ++j)
      for (int i = 0; i <= ny + 1; ++i) {
        cn[IX(i, j, 0)] = cn[IX(i, j, 1)];
        cn[IX(i, j, nz + 1)] = cn[IX(i, j, nz)];
      }
  }
  free(div);
}

/* The per-frame body of the AccDiff_3D program, AD:76-243: psi from the
 * distance field with width `width` (0.75 at AD:84), Neumann ghosts, the
 * solid sweep, then the electrolyte sweep on psi = 1 - psi (interior only;
 * the ghosts keep the solid values, AD:175). */
void orc_connectivity(int py, int px, int pz, const double* dist, double width,
                      int term, double* cn_solid, double* cn_elec) {
  const int ny = py, nx = px, nz = pz;
  double* psi = (double*)calloc(NH, sizeof(double));
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const double d = dist[(size_t)(i - 1) + (size_t)ny * ((size_t)(j - 1) + (size_t)nx * (size_t)(k - 1))];
        psi[IX(i, j, k)] = 0.5 * (1.0 + tanh(d / width));
      }
  orc_nogrdbc(py, px, pz, psi); /* AD:88-97 is the same fill */
  memset(cn_solid, 0, NH * sizeof(double));
  orc_accdiff(py, px, pz, psi, cn_solid, term, 1);
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) psi[IX(i, j, k)] = 1.0 - psi[IX(i, j, k)];
  memset(cn_elec, 0, NH * sizeof(double));
  orc_accdiff(py, px, pz, psi, cn_elec, term, 0);
  free(psi);
}

/* The per-frame body of the RM_UCNCT_3D program, RM:68-141 (both phases):
 * psA = 0.5*(1.0+TANH(d/1.0)) (electrolyte: 1 - psA), psB = psA with 0
 * where the phase's Cn < 1.0e-4 (REAL(4)), dsF = psB with NoGrdBc3D
 * ghosts, sign (> 0.5), reinitialisation from zero for `lit` steps with
 * dt = 1.0e-1 REAL(4).  cn_* and dist are interior arrays; d_* halo-padded. */
void orc_rm_ucnct(int py, int px, int pz, const double* dist, const double* cn_solid,
                  const double* cn_elec, int lit, double* d_solid, double* d_elec) {
  const int ny = py, nx = px, nz = pz;
  const size_t n = (size_t)ny * nx * nz;
  const double thr = (double)1.0e-4f;
  double* psa = (double*)malloc(n * sizeof(double));
  double* sg = (double*)malloc(NH * sizeof(double));
  for (size_t c = 0; c < n; ++c) psa[c] = 0.5 * (1.0 + tanh(dist[c] / 1.0));
  for (int phase = 0; phase < 2; ++phase) {
    const double* cn = phase == 0 ? cn_solid : cn_elec;
    double* ds = phase == 0 ? d_solid : d_elec;
    if (phase == 1)
      for (size_t c = 0; c < n; ++c) psa[c] = 1.0e0 - psa[c];
    memset(ds, 0, NH * sizeof(double));
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const size_t q = (size_t)(i - 1) + (size_t)ny * ((size_t)(j - 1) + (size_t)nx * (k - 1));
          ds[IX(i, j, k)] = (cn[q] < thr) ? 0.0 : psa[q];
        }
    orc_nogrdbc(py, px, pz, ds);
    orc_sign((int64_t)NH, ds, 0.5, sg);
    memset(ds, 0, NH * sizeof(double));
    orc_redist(lit, (double)1.0e-1f, py, px, pz, sg, ds);
  }
  free(psa);
  free(sg);
}

/* RM:79-82 and RM:119,128-130. */
void orc_rm_mask(int64_t n, const double* psA, const double* cn, double* psB) {
  const double thr = (double)1.0e-4f;
  for (int64_t c = 0; c < n; ++c) psB[c] = (cn[c] < thr) ? 0.0 : psA[c];
}

/* LS:140-144, RM:92-96. */
void orc_sign(int64_t n, const double* ds, double thr, double* sg) {
  for (int64_t c = 0; c < n; ++c) sg[c] = (ds[c] > thr) ? 1.0 : -1.0;
}

/* ---------------------------------------------------------------- fields */

/* SBMES:154-168 then the single-rank halo (BcMpiYZ + x lines, :173-176),
 * which on one rank equals the edge-copy fill of NoGrdBc3D. */
void orc_psi_from_dist(int ny, int nx, int nz, const float* d, double zeta, double* psi) {
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        double v = (double)d[(size_t)(i - 1) + (size_t)ny * ((size_t)(j - 1) + (size_t)nx * (size_t)(k - 1))];
        v = 0.5 * (1.0 + tanh(v / zeta));
        if (v < 0.0) v = 0.0;
        if (v > 1.0) v = 1.0;
        psi[IX(i, j, k)] = v;
      }
  orc_nogrdbc(ny, nx, nz, psi);
}

/* SBMES:273-291. */
void orc_avp(int ny, int nx, int nz, const double* psP, const double* psE, double dx,
             double mask, double* avp, double* avpx) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        double a = (psP[IX(i + 1, j, k)] - psP[IX(i - 1, j, k)]) / 2.0;
        double b = (psP[IX(i, j + 1, k)] - psP[IX(i, j - 1, k)]) / 2.0;
        double e = (psP[IX(i, j, k + 1)] - psP[IX(i, j, k - 1)]) / 2.0;
        const double gp = sqrt((a * a + b * b) + e * e);
        a = (psE[IX(i + 1, j, k)] - psE[IX(i - 1, j, k)]) / 2.0;
        b = (psE[IX(i, j + 1, k)] - psE[IX(i, j - 1, k)]) / 2.0;
        e = (psE[IX(i, j, k + 1)] - psE[IX(i, j, k - 1)]) / 2.0;
        const double ge = sqrt((a * a + b * b) + e * e);
        double v = sqrt(gp * ge);
        if (v < mask) v = 0.0;
        avp[c] = v;
        avpx[c] = v / dx;
      }
}

/* Tbl_Chk_Pln_3DA, SBMES:987-1028, including its one-segment-left index
 * (lb = FLOOR(c/ditv) addresses Cord(lb), which is (lb-1)*ditv). */
void orc_table(int64_t n, int sz, const double* cord, const double* vals,
               const double* cn, double* fn) {
  const double ditv = cord[1] - cord[0];
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < n; ++c) {
    double t = cn[c];
    if (t < 0.0) t = 1.0e-6;
    if (t > 1.0) t = 1.0;
    const double fl = floor(t / ditv);
    int lb = (fl >= 0.0 && fl < 2147483647.0) ? (int)fl : 0;
    if (lb == 0) lb = 1;
    else if (lb == sz) lb = sz - 1;
    /* beyond the table the reference reads outside its arrays; stay inside */
    if (lb > sz - 1) lb = sz - 1;
    fn[c] = vals[lb - 1] + ((t - cord[lb - 1]) / ditv) * (vals[lb] - vals[lb - 1]);
  }
}

/* ------------------------------------------------------------- operator */

/* S = sum over faces of c_f (p_nb - p_c) with c_f = (K_nb + K_c)*0.5, in
 * the term order of SBMES:494-499 (y+, y-, x+, x-, z+, z-). */
static inline double sbm_S(int ny, int nx, const double* K, const double* p,
                           int i, int j, int k) {
  (void)0;
  const size_t c = IX(i, j, k);
  const double kc = K[c], pc = p[c];
  const size_t ym = IX(i - 1, j, k), yp = IX(i + 1, j, k);
  const size_t xm = IX(i, j - 1, k), xp = IX(i, j + 1, k);
  const size_t zm = IX(i, j, k - 1), zp = IX(i, j, k + 1);
  const double c1 = (K[ym] + kc) * 0.5, c2 = (K[yp] + kc) * 0.5;
  const double c3 = (K[xm] + kc) * 0.5, c4 = (K[xp] + kc) * 0.5;
  const double c5 = (K[zm] + kc) * 0.5, c6 = (K[zp] + kc) * 0.5;
  double s = c2 * (p[yp] - pc);
  s = s - c1 * (pc - p[ym]);
  s = s + c4 * (p[xp] - pc);
  s = s - c3 * (pc - p[xm]);
  s = s + c6 * (p[zp] - pc);
  s = s - c5 * (pc - p[zm]);
  return s;
}

/* q = diag*p - scale*S(p)  (CnE form, SBMES:515-521) when diag != NULL,
 * q = scale*S(p)           (phP/phE form, SBMES:670-676) otherwise.
 * p's ghosts are read as stored. */
void orc_apply(int ny, int nx, int nz, const double* K, const double* diag,
               double scale, const double* p, double* q) {
  (void)nz;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double s = sbm_S(ny, nx, K, p, i, j, k);
        q[c] = diag ? diag[c] * p[c] - scale * s : scale * s;
      }
}

/* RES = RHS - A x with x's stored ghosts (SBMES:492-499, :649-655, :729-735). */
void orc_residual(int ny, int nx, int nz, const double* K, const double* diag,
                  double scale, const double* rhs, const double* x, double* r) {
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double s = sbm_S(ny, nx, K, x, i, j, k);
        const double ax = diag ? diag[c] * x[c] - scale * s : scale * s;
        r[c] = rhs[c] - ax;
      }
}

/* The reference CG loop (SBMES:501-554 CnE, :657-714 phP, :737-795 phE):
 * unpreconditioned CG with the search-direction ghost rules bc_x0/bc_x1
 * (SBM_BC_COPY / SBM_BC_ZERO) and y/z edge copies.  Executes at most
 * max_it iterations (the reference's `IF (itlp > cap) EXIT` runs cap+1). */
int orc_cg(int ny, int nx, int nz, const double* K, const double* diag, double scale,
           int bc_x0, int bc_x1, const double* rhs, double* x, const double* w,
           double wsum, int stop_rule, double tol, int max_it,
           int* iters, double* final_res) {
  const size_t n = NH;
  double* res = (double*)calloc(n, sizeof(double));
  double* prj = (double*)calloc(n, sizeof(double));
  double* wmx = (double*)calloc(n, sizeof(double));
  double* tmp = (double*)calloc(n, sizeof(double));
  orc_residual(ny, nx, nz, K, diag, scale, rhs, x, res);
  memcpy(prj, res, n * sizeof(double));
  const double rr0 = sum_sq_w(ny, nx, nz, res, NULL);
  double rms = 1.0;
  int it = 0, status = SBM_ERR_MAXIT;
  if (stop_rule == SBM_STOP_REL_RES && rr0 == 0.0) {
    status = SBM_OK;
    rms = 0.0;
  } else {
    while (it < max_it) {
      if (stop_rule == SBM_STOP_REF_UPDATE) memcpy(tmp, x, n * sizeof(double));
      orc_bc_yz(ny, nx, nz, prj);
      orc_bc_x(ny, nx, nz, prj, 0, nz + 1, bc_x0, 0.0, bc_x1, 0.0);
      orc_apply(ny, nx, nz, K, diag, scale, prj, wmx);
      const double dmy = sum_sq_w(ny, nx, nz, res, NULL);
      const double btm = sum_prod(ny, nx, nz, prj, wmx);
      const double alp = dmy / btm;
#pragma omp parallel for schedule(static)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= nx; ++j)
          for (int i = 1; i <= ny; ++i) {
            const size_t c = IX(i, j, k);
            x[c] = x[c] + alp * prj[c];
            res[c] = res[c] - alp * wmx[c];
          }
      const double btm2 = sum_sq_w(ny, nx, nz, res, NULL);
      const double bet = btm2 / dmy;
#pragma omp parallel for schedule(static)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= nx; ++j)
          for (int i = 1; i <= ny; ++i) {
            const size_t c = IX(i, j, k);
            prj[c] = res[c] + bet * prj[c];
          }
      ++it;
      if (stop_rule == SBM_STOP_REF_UPDATE)
        rms = sqrt(sum_dsq_w(ny, nx, nz, x, tmp, w) / wsum);
      else if (stop_rule == SBM_STOP_REF_RESID)
        rms = sqrt(sum_sq_w(ny, nx, nz, res, w) / wsum);
      else
        rms = sqrt(btm2) / sqrt(rr0);
      if (!isfinite(rms) || !isfinite(alp)) {
        status = SBM_ERR_NONFINITE;
        break;
      }
      if (!(rms > tol)) {
        status = SBM_OK;
        break;
      }
    }
  }
  if (iters) *iters = it;
  if (final_res) *final_res = rms;
  free(res);
  free(prj);
  free(wmx);
  free(tmp);
  return status;
}

/* ------------------------------------------------------- reference params */

/* The reference's parameters and literal values (SBMES:90-136), REAL(4)
 * literals promoted as Fortran does. */
int orc_params_reference(sbm_params* p) {
  if (!p) return SBM_ERR_ARG;
  memset(p, 0, sizeof(*p));
  p->dx = 3.25e-5 * 0.5;                               /* SBMES:90 */
  p->rho = (double)0.0312f;                             /* SBMES:100 */
  p->eps = 6.7600e-10;                                  /* SBMES:136 */
  p->ch_mask = 1.0e-5;                                  /* SBMES:430 */
  p->cst1 = 1.6021766e-19 / (1.3806488e-23 * 300.0);   /* SBMES:101 */
  p->frd = (double)96485.3365f;                         /* SBMES:102 */
  p->bvp = (double)(-0.1f);                             /* SBMES:106 */
  p->bve = (double)(-0.4495f);                          /* SBMES:107 */
  const double de = 2.0 * (4.0e-6 * 1.25e-6) / (4.0e-6 + 1.25e-6); /* :118 */
  p->t_minus = 4.0e-6 / (4.0e-6 + 1.25e-6);                     /* :121 */
  p->d0 = (de / 2.598606299407882e-06) * (double)0.006667f;     /* :124 */
  p->tc1 = (2 * p->t_minus - 1.0) / (2 * p->t_minus * (1.0 - p->t_minus)); /* :125 */
  p->tc2 = 1.0 / (2 * p->t_minus * (1.0 - p->t_minus)) * p->cst1;         /* :126 */
  p->dab_c0 = (double)(-7.02f);                         /* :474 */
  p->dab_c1 = 0.83e3;   /* subtracted: c0 - c1*c + c2*(c3*c)**2 */
  p->dab_c2 = (double)0.05f;
  p->dab_c3 = 1.0e3;
  p->cne_ref = 1.0e-3;                                  /* :567 */
  p->kap_scale = (double)3.3f;                          /* :324 */
  p->avp_mask = 1.0e-2;                                 /* :287, :631 */
  p->i0_scale = 1.0e-3;                                 /* :617 */
  p->kfw_c = (double)0.001f;                            /* :621 */
  p->crt_cne = 1.0e-7;                                  /* :96 */
  p->crt_php = 1.0e-7;                                  /* :97 */
  p->crt_phe = 1.0e-6;                                  /* :98 */
  p->crt_picard = 1.0e-8;                               /* :627 */
  p->max_it_cne = 50001;                                /* :551 */
  p->max_it_php = 30001;                                /* :710 */
  p->max_it_phe = 100001;                               /* :791 */
  p->max_picard = 1000;
  p->cne_mean_every = 100;                              /* :562 */
  p->bv_mode = SBM_BV_EXP;
  p->ch_mode = SBM_CH_TABLE;
  p->ch_w = 1.0;
  p->tbl_n = 101;
  for (int t = 0; t < 101; ++t) {
    p->tbl_x[t] = t * 0.01;
    p->tbl_mu[t] = 0.0;
    p->tbl_mb[t] = 0.0;
    p->tbl_i0[t] = 0.0;
    p->tbl_ocv[t] = 0.0;
  }
  return SBM_OK;
}

/* ------------------------------------------------------ electrochem state */

struct orc_state {
  int ny, nx, nz;
  sbm_params p;
  double tPP, tPE, xrf, infx, scrnt, trgI, bve;
  double* f[SBM_F_COUNT];
  /* work fields, all halo-padded */
  double *lap, *mu, *mb, *pmN, *dab, *dab1, *pce, *pcc, *kap, *rhs, *rhe, *rxc,
      *kfw, *kbw, *ppo, *peo, *tmpf;
};

orc_state* orc_state_new(int ny, int nx, int nz, const sbm_params* p) {
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  s->ny = ny;
  s->nx = nx;
  s->nz = nz;
  s->p = *p;
  const size_t n = NH;
  for (int f = 0; f < SBM_F_COUNT; ++f) s->f[f] = (double*)calloc(n, sizeof(double));
  double** w[] = {&s->lap, &s->mu, &s->mb, &s->pmN, &s->dab, &s->dab1, &s->pce, &s->pcc,
                  &s->kap, &s->rhs, &s->rhe, &s->rxc, &s->kfw, &s->kbw, &s->ppo, &s->peo,
                  &s->tmpf};
  for (size_t t = 0; t < sizeof(w) / sizeof(w[0]); ++t) *w[t] = (double*)calloc(n, sizeof(double));
  return s;
}

void orc_state_free(orc_state* s) {
  if (!s) return;
  for (int f = 0; f < SBM_F_COUNT; ++f) free(s->f[f]);
  double* w[] = {s->lap, s->mu, s->mb, s->pmN, s->dab, s->dab1, s->pce, s->pcc,
                 s->kap, s->rhs, s->rhe, s->rxc, s->kfw, s->kbw, s->ppo, s->peo, s->tmpf};
  for (size_t t = 0; t < sizeof(w) / sizeof(w[0]); ++t) free(w[t]);
  free(s);
}

double* orc_state_field(orc_state* s, int field) {
  if (field >= 0 && field < SBM_F_COUNT) return s->f[field];
  return NULL;
}

static void fill_scalars(orc_state* s, sbm_scalars* sc) {
  if (!sc) return;
  sc->tPP = s->tPP;
  sc->tPE = s->tPE;
  sc->xrf = s->xrf;
  sc->infx = s->infx;
  sc->scrnt = s->scrnt;
  sc->trgI = s->trgI;
  sc->bve = s->bve;
}

/* SBMES:154-341 for one rank that owns the whole grid. */
int orc_setup_domain(orc_state* s, const float* dist_p, const float* dist_e,
                     double zeta, double cnp0, double cne0, double cr, sbm_scalars* sc) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const size_t n = NH;
  double *psP = s->f[SBM_F_PSP], *psE = s->f[SBM_F_PSE];
  orc_psi_from_dist(ny, nx, nz, dist_p, zeta, psP);
  orc_psi_from_dist(ny, nx, nz, dist_e, zeta, psE);
  for (size_t c = 0; c < n; ++c) psP[c] = psP[c] + 1.0e-7;   /* :247 */
  s->tPP = sum_prod(ny, nx, nz, psP, NULL);                  /* :248-252 */
  for (size_t c = 0; c < n; ++c) psE[c] = psE[c] + 1.0e-6;   /* :258 */
  s->tPE = sum_prod(ny, nx, nz, psE, NULL);                  /* :260-262 */
  orc_avp(ny, nx, nz, psP, psE, s->p.dx, s->p.avp_mask, s->f[SBM_F_AVP], s->f[SBM_F_AVPX]);
  for (size_t c = 0; c < n; ++c) {
    s->f[SBM_F_CNP][c] = cnp0;                               /* :297 */
    s->f[SBM_F_CNE][c] = cne0;                               /* :307 */
    s->f[SBM_F_RXN][c] = 0.0;                                /* :313 */
    s->f[SBM_F_PHP][c] = s->p.bvp;                           /* :318 */
    s->f[SBM_F_PHE][c] = s->p.bve;                           /* :337 */
    s->kap[c] = s->p.kap_scale * psP[c];                     /* :324 */
    s->rxc[c] = 0.0;
  }
  s->xrf = sum_prod(ny, nx, nz, s->f[SBM_F_CNP], psP) / s->tPP; /* :301-303 */
  s->trgI = (((double)0.95f * s->tPP) * s->p.rho) / (3600 / cr); /* :341 */
  s->scrnt = s->trgI;                                         /* :351 */
  s->bve = s->p.bve;
  s->infx = 0.0;
  fill_scalars(s, sc);
  return SBM_OK;
}

/* edge-copy halo of BcMpiYZ + the x lines that copy, SBMES:407-409 etc. */
static void bc_copy_all(int ny, int nx, int nz, double* f) {
  orc_bc_yz(ny, nx, nz, f);
  orc_bc_x(ny, nx, nz, f, 0, nz + 1, 0, 0.0, 0, 0.0);
}

/* Cahn-Hilliard update of CnP, SBMES:397-443. */
int orc_ch_step(orc_state* s, double dt, sbm_scalars* sc) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const sbm_params* p = &s->p;
  double *cnp = s->f[SBM_F_CNP], *psP = s->f[SBM_F_PSP];
  const double dx2 = p->dx * p->dx;
  /* :398-400 */
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double u = cnp[c];
        double t = cnp[IX(i, j - 1, k)] - 2.0 * u;
        t = t + cnp[IX(i, j + 1, k)];
        t = t + cnp[IX(i - 1, j, k)];
        t = t - 2.0 * u;
        t = t + cnp[IX(i + 1, j, k)];
        t = t + cnp[IX(i, j, k - 1)];
        t = t - 2.0 * u;
        t = t + cnp[IX(i, j, k + 1)];
        s->lap[c] = t / dx2;
      }
  /* :403, :405 table lookups on the interior */
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j) {
      const size_t c0 = IX(1, j, k);
      orc_table(ny, p->tbl_n, p->tbl_x, p->tbl_mu, cnp + c0, s->mu + c0);
      orc_table(ny, p->tbl_n, p->tbl_x, p->tbl_mb, cnp + c0, s->mb + c0);
      if (p->ch_mode == SBM_CH_DOUBLE_WELL)
        for (int i = 1; i <= ny; ++i) { /* mu = W*2*c*(1-c)*(1-2*c), left to right */
          const double u = cnp[c0 + i - 1];
          s->mu[c0 + i - 1] = (((p->ch_w * 2.0) * u) * (1.0 - u)) * (1.0 - 2.0 * u);
        }
    }
  bc_copy_all(ny, nx, nz, s->mb);                             /* :407-409 */
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        s->mu[c] = s->mu[c] - p->eps * s->lap[c];             /* :411 */
      }
  bc_copy_all(ny, nx, nz, s->mu);                             /* :413-415 */
  for (size_t c = 0; c < NH; ++c) s->pmN[c] = psP[c] * s->mb[c]; /* :419 */
  double* dvc = s->tmpf;
  const double* pm = s->pmN;
  const double* mu = s->mu;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {                         /* :422-428 */
        const size_t c = IX(i, j, k);
        const size_t ym = IX(i - 1, j, k), yp = IX(i + 1, j, k);
        const size_t xm = IX(i, j - 1, k), xp = IX(i, j + 1, k);
        const size_t zm = IX(i, j, k - 1), zp = IX(i, j, k + 1);
        double t = (0.5 * (pm[yp] + pm[c])) * (mu[yp] - mu[c]);
        t = t - (0.5 * (pm[c] + pm[ym])) * (mu[c] - mu[ym]);
        t = t + ((1.0 * 0.5) * (pm[xp] + pm[c])) * (mu[xp] - mu[c]);
        t = t - ((1.0 * 0.5) * (pm[c] + pm[xm])) * (mu[c] - mu[xm]);
        t = t + (0.5 * (pm[zp] + pm[c])) * (mu[zp] - mu[c]);
        t = t - (0.5 * (pm[c] + pm[zm])) * (mu[c] - mu[zm]);
        dvc[c] = t / dx2;
      }
  const double* rxn = s->f[SBM_F_RXN];
  const double* avpx = s->f[SBM_F_AVPX];
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {                         /* :430-433 */
        const size_t c = IX(i, j, k);
        if (psP[c] > p->ch_mask)
          cnp[c] = cnp[c] + (dt * (dvc[c] + (rxn[c] / p->rho) * avpx[c])) / psP[c];
      }
  bc_copy_all(ny, nx, nz, cnp);                               /* :436-438 */
  s->xrf = sum_prod(ny, nx, nz, cnp, psP) / s->tPP;          /* :441-443 */
  fill_scalars(s, sc);
  return SBM_OK;
}

/* Dab = scale*D0*EXP(c0 - c1*c + c2*(c3*c)**2) over the whole padded
 * array (SBMES:474, :579, :601); a scaled Dab multiplies as (scale*D0). */
static void dab_fill(orc_state* s, double scale, int scaled, double* out) {
  const sbm_params* p = &s->p;
  const double* cne = s->f[SBM_F_CNE];
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const double pre = scaled ? scale * p->d0 : p->d0;
#pragma omp parallel for schedule(static)
  for (long long c = 0; c < (long long)NH; ++c) {
    const double u = cne[c];
    const double q = p->dab_c3 * u;
    out[c] = pre * exp((p->dab_c0 - p->dab_c1 * u) + p->dab_c2 * (q * q));
  }
}

static void cne_flux_bc(orc_state* s) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  double* cne = s->f[SBM_F_CNE];
  const double* dab = s->dab;
  orc_bc_yz(ny, nx, nz, cne);                                 /* :557 */
  for (int k = 0; k <= nz + 1; ++k)
    for (int i = 0; i <= ny + 1; ++i) {                       /* :558, :560 */
      cne[IX(i, 0, k)] = ((s->infx * s->p.t_minus) * s->p.dx) /
                             (0.5 * (dab[IX(i, 0, k)] + dab[IX(i, 1, k)])) +
                         cne[IX(i, 1, k)];
      cne[IX(i, nx + 1, k)] = cne[IX(i, nx, k)];
    }
}

/* Electrolyte concentration, SBMES:461-572. */
int orc_cne_step(orc_state* s, int iter, double dt, sbm_scalars* sc) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const sbm_params* p = &s->p;
  double *cne = s->f[SBM_F_CNE], *psE = s->f[SBM_F_PSE];
  const double *rxn = s->f[SBM_F_RXN], *avpx = s->f[SBM_F_AVPX];
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) {                         /* :461-462 */
        const size_t c = IX(i, j, k);
        s->rhs[c] = psE[c] * cne[c] - ((dt * rxn[c]) * avpx[c]) * p->t_minus;
      }
  /* :465-467 */
  const double lsm = sum_prod(ny, nx, nz, rxn, avpx) * ((p->dx * p->dx) * p->dx);
  s->infx = lsm / ((double)(ny * nz) * (p->dx * p->dx));
  dab_fill(s, 1.0, 0, s->dab);                                /* :474 */
  for (size_t c = 0; c < NH; ++c) s->pce[c] = psE[c] * s->dab[c]; /* :478-484 */
  const double scale = dt / (p->dx * p->dx);
  int it = 0;
  double rms = 0.0;
  int st = SBM_OK;
  if (iter > 1) {                                             /* :505-555 */
    st = orc_cg(ny, nx, nz, s->pce, psE, scale, SBM_BC_COPY, SBM_BC_COPY, s->rhs, cne, psE,
                s->tPE, SBM_STOP_REF_RESID, p->crt_cne, p->max_it_cne, &it, &rms);
  }
  cne_flux_bc(s);
  if (iter % p->cne_mean_every == 1) {                        /* :562-572 */
    const double av = sum_prod(ny, nx, nz, psE, cne) / s->tPE;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) cne[IX(i, j, k)] = cne[IX(i, j, k)] - (av - p->cne_ref);
    cne_flux_bc(s);
  }
  if (sc) {
    fill_scalars(s, sc);
    sc->it_cne = it;
  }
  return st == SBM_ERR_MAXIT ? SBM_OK : st;
}

/* Potentials with the Butler-Volmer Picard loop, SBMES:577-812. */
int orc_bv_update(orc_state* s, sbm_scalars* sc) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  const sbm_params* p = &s->p;
  double *cne = s->f[SBM_F_CNE], *cnp = s->f[SBM_F_CNP], *psE = s->f[SBM_F_PSE];
  double *psP = s->f[SBM_F_PSP], *php = s->f[SBM_F_PHP], *phe = s->f[SBM_F_PHE];
  double *rxn = s->f[SBM_F_RXN], *avp = s->f[SBM_F_AVP], *avpx = s->f[SBM_F_AVPX];
  const double idx2 = 1.0 / (p->dx * p->dx);
  /* :579-596 */
  dab_fill(s, p->tc1, 1, s->dab1);
  for (size_t c = 0; c < NH; ++c) s->pce[c] = psE[c] * s->dab1[c];
  orc_apply(ny, nx, nz, s->pce, NULL, idx2, cne, s->rhe);
  /* :601-610 */
  dab_fill(s, p->tc2, 1, s->dab1);
  for (size_t c = 0; c < NH; ++c) s->pcc[c] = (psE[c] * cne[c]) * s->dab1[c];
  /* :614-622 */
  const double ac = 0.5 * p->cst1;
#pragma omp parallel for schedule(static)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j) {
      const size_t c0 = IX(1, j, k);
      orc_table(ny, p->tbl_n, p->tbl_x, p->tbl_i0, cnp + c0, s->kfw + c0);
      orc_table(ny, p->tbl_n, p->tbl_x, p->tbl_ocv, cnp + c0, s->kbw + c0);
      for (int i = 1; i <= ny; ++i) {
        const size_t c = IX(i, j, k);
        const double ioc = s->kfw[c] * p->i0_scale;
        const double ocv = s->kbw[c];
        s->kfw[c] = (ioc / (p->frd * p->kfw_c)) * exp(ac * ocv);
        s->kbw[c] = (ioc / (p->frd * cnp[c])) * exp(-(ac * ocv));
      }
    }
  double cvgp = 1.0, cvgl = 1.0;
  int nlp = 0, itp = 0, ite = 0;
  int st = SBM_OK;
  while (cvgp > p->crt_picard && cvgl > p->crt_picard && nlp < p->max_picard) {
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {                       /* :631-641 */
          const size_t c = IX(i, j, k);
          if (avp[c] > p->avp_mask) {
            const double dph = php[c] - phe[c];
            double r;
            if (p->bv_mode == SBM_BV_LINEAR)
              r = (s->kfw[c] * cne[c]) * (1.0 - ac * dph) - (s->kbw[c] * cnp[c]) * (1.0 + ac * dph);
            else
              r = (s->kfw[c] * cne[c]) * exp(-(ac * dph)) - (s->kbw[c] * cnp[c]) * exp(ac * dph);
            rxn[c] = r;
            s->rxc[c] = r * p->frd;
          }
        }
    /* phP, :644-723 */
    memcpy(s->ppo, php, NH * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const size_t c = IX(i, j, k);
          s->rhs[c] = -s->rxc[c] * avpx[c];
        }
    for (int k = 0; k <= nz + 1; ++k)
      for (int i = 0; i <= ny + 1; ++i) php[IX(i, nx + 1, k)] = p->bvp;
    int it = 0;
    double rms = 0.0;
    int r1 = orc_cg(ny, nx, nz, s->kap, NULL, idx2, SBM_BC_COPY, SBM_BC_ZERO, s->rhs, php,
                    psP, s->tPP, SBM_STOP_REF_UPDATE, p->crt_php, p->max_it_php, &it, &rms);
    itp = it;
    orc_bc_yz(ny, nx, nz, php);
    orc_bc_x(ny, nx, nz, php, 0, nz + 1, 0, 0.0, 1, p->bvp);
    cvgp = sqrt(sum_dsq_w(ny, nx, nz, php, s->ppo, psP) / s->tPP);
    /* phE, :726-804 */
    memcpy(s->peo, phe, NH * sizeof(double));
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= nx; ++j)
        for (int i = 1; i <= ny; ++i) {
          const size_t c = IX(i, j, k);
          s->rhs[c] = rxn[c] * avpx[c] + s->rhe[c];
        }
    int r2 = orc_cg(ny, nx, nz, s->pcc, NULL, idx2, SBM_BC_ZERO, SBM_BC_COPY, s->rhs, phe,
                    psE, s->tPE, SBM_STOP_REF_UPDATE, p->crt_phe, p->max_it_phe, &it, &rms);
    ite = it;
    orc_bc_yz(ny, nx, nz, phe);
    orc_bc_x(ny, nx, nz, phe, 0, nz + 1, 1, s->bve, 0, 0.0);
    cvgl = sqrt(sum_dsq_w(ny, nx, nz, phe, s->peo, psE) / s->tPE);
    ++nlp;
    if (r1 == SBM_ERR_NONFINITE || r2 == SBM_ERR_NONFINITE) {
      st = SBM_ERR_NONFINITE;
      break;
    }
  }
  if (sc) {
    fill_scalars(s, sc);
    sc->cvgp = cvgp;
    sc->cvgl = cvgl;
    sc->it_php = itp;
    sc->it_phe = ite;
    sc->n_picard = nlp;
  }
  return st;
}

/* Current and voltage control, SBMES:826-835. */
int orc_voltage_step(orc_state* s, double dt, double vsr, sbm_scalars* sc) {
  const int ny = s->ny, nx = s->nx, nz = s->nz;
  double* phe = s->f[SBM_F_PHE];
  s->scrnt = sum_prod(ny, nx, nz, s->f[SBM_F_RXN], s->f[SBM_F_AVPX]);
  const double d = s->trgI - s->scrnt;
  const double sv = copysign(fabs(vsr), d); /* DSIGN: the sign of d, -0.0 negative */
  s->bve = s->bve + sv * dt;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= nx; ++j)
      for (int i = 1; i <= ny; ++i) phe[IX(i, j, k)] = phe[IX(i, j, k)] + sv * dt;
  orc_bc_yz(ny, nx, nz, phe);
  orc_bc_x(ny, nx, nz, phe, 1, nz, 1, s->bve, 0, 0.0);
  fill_scalars(s, sc);
  return SBM_OK;
}

/* One pass of the reference's time loop body, DO WHILE (Xrf < 0.971)
 * (SBMES:357-877): Cahn-Hilliard, the CnE solve, the Butler-Volmer Picard
 * loop with the phP / phE solves, and the voltage control. */
int orc_time_step(orc_state* s, int iter, double dt, double vsr, sbm_scalars* sc) {
  sbm_scalars tmp;
  memset(&tmp, 0, sizeof(tmp));
  int st = orc_ch_step(s, dt, &tmp);
  if (st) return st;
  st = orc_cne_step(s, iter, dt, &tmp);
  if (st) return st;
  const int it_cne = tmp.it_cne;
  st = orc_bv_update(s, &tmp);
  if (st) return st;
  st = orc_voltage_step(s, dt, vsr, &tmp);
  tmp.it_cne = it_cne;
  if (sc) *sc = tmp;
  return st;
}
