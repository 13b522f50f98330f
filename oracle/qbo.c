/* qbo.c -- CPU FP64 oracle for the qball H|psi> / ETRS hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see qbo.h).  Compiled with -ffp-contract=off so
 * that every product and sum is rounded separately, as in the reference's
 * x86 build, and so that this file gives the same bits on x86 and aarch64.
 * Complex arithmetic is spelled out as (ac-bd, ad+bc), the same sequence as
 * the libgcc complex multiply the reference's std::complex<double> uses.
 */
#include "qbo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* Unit cell: UnitCell::set (UnitCell.cc:37-100) and D3vector (d3vector.h)  */
/* ------------------------------------------------------------------------ */
static void cross3(const double* a, const double* b, double* c) {
  /* d3vector.h operator^ */
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

double qbo_cell_volume(const double* a) {
  double c[3];
  cross3(a + 3, a + 6, c);
  return a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
}

void qbo_cell_b(const double* a, double* b) {
  /* amt0 = (fac*a1)^a2, amt1 = (fac*a2)^a0, amt2 = (fac*a0)^a1,
   * b_i = (2 pi) * amt_i  (UnitCell.cc:52-78) */
  const double vol = qbo_cell_volume(a);
  if (!(vol > 0.0)) {
    memset(b, 0, 9 * sizeof(double));
    return;
  }
  const double fac = 1.0 / vol;
  const double twopi = 2.0 * M_PI;
  for (int i = 0; i < 3; ++i) {
    const double* p = a + 3 * ((i + 1) % 3);
    const double* q = a + 3 * ((i + 2) % 3);
    double fp[3] = {p[0] * fac, p[1] * fac, p[2] * fac};
    double c[3];
    cross3(fp, q, c);
    for (int j = 0; j < 3; ++j) b[3 * i + j] = c[j] * twopi;
  }
}

/* Basis::factorizable (Basis.cc:126-150): 2^h 3^i 5^j 7^k 11^m, i<=2, j,k,m<=1 */
int qbo_factorizable(int n) {
  if (n % 11 == 0) n /= 11;
  if (n % 7 == 0) n /= 7;
  if (n % 5 == 0) n /= 5;
  if (n % 3 == 0) n /= 3;
  if (n % 3 == 0) n /= 3;
  while (n % 2 == 0) n /= 2;
  return n == 1;
}

/* ------------------------------------------------------------------------ */
/* Basis::resize, complex (force_complex) branch at k=0 with one process     */
/* (Basis.cc:302-700).  Rods are kept in the reference's multiset order:     */
/* ascending size, ties in generation order (h outer, k inner), then rod     */
/* (0,0) swapped with the first rod (Basis.cc:640-660).                      */
/* ------------------------------------------------------------------------ */
typedef struct {
  int h, k, lmin, size;
} qbo_rod;

static int qbo_build_rods(const double* a, double ecut, qbo_rod** rods_out,
                          int* info) {
  double b[9];
  qbo_cell_b(a, b);
  const double two_ecut = 2.0 * ecut;
  const double twopi = 2.0 * M_PI;
  const double fac = sqrt(two_ecut) / twopi;
  const double la0 = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double la1 = sqrt(a[3] * a[3] + a[4] * a[4] + a[5] * a[5]);
  const double la2 = sqrt(a[6] * a[6] + a[7] * a[7] + a[8] * a[8]);
  const int hmax = (int)(0.5 + fac * la0), hmin = -hmax;
  const int kmax = (int)(0.5 + fac * la1), kmin = -kmax;
  const int lmax = (int)(0.5 + fac * la2), lmin = -lmax;

  int cap = (hmax - hmin + 3) * (kmax - kmin + 3);
  qbo_rod* rods = (qbo_rod*)malloc(sizeof(qbo_rod) * (size_t)cap);
  int nrods = 0, size = 0;
  int hmax_used = hmin, hmin_used = hmax, kmax_used = kmin, kmin_used = kmax;
  int lmax_used = lmin, lmin_used = lmax;
  for (int h = hmin - 1; h <= hmax + 1; ++h) {
    for (int k = kmin - 1; k <= kmax + 1; ++k) {
      int lstart = lmax, lend = lmin, found = 0;
      for (int l = lmin - 1; l <= lmax + 1; ++l) {
        /* norm((kpx+h)*b0 + (kpy+k)*b1 + (kpz+l)*b2), k-point = 0 */
        const double dh = 0.0 + h, dk = 0.0 + k, dl = 0.0 + l;
        double v[3];
        for (int j = 0; j < 3; ++j)
          v[j] = (b[j] * dh + b[3 + j] * dk) + b[6 + j] * dl;
        const double two_e = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        if (two_e < two_ecut) {
          if (l < lstart) lstart = l;
          if (l > lend) lend = l;
          found = 1;
        }
      }
      if (found) {
        const int rodsize = lend - lstart + 1;
        size += rodsize;
        rods[nrods].h = h;
        rods[nrods].k = k;
        rods[nrods].lmin = lstart;
        rods[nrods].size = rodsize;
        ++nrods;
        if (h > hmax_used) hmax_used = h;
        if (h < hmin_used) hmin_used = h;
        if (k > kmax_used) kmax_used = k;
        if (k < kmin_used) kmin_used = k;
        if (lend > lmax_used) lmax_used = lend;
        if (lstart < lmin_used) lmin_used = lstart;
      }
    }
  }
  /* stable sort by size (multiset<Rod> keeps insertion order among equals) */
  for (int i = 1; i < nrods; ++i) {
    qbo_rod r = rods[i];
    int j = i - 1;
    while (j >= 0 && rods[j].size > r.size) {
      rods[j + 1] = rods[j];
      --j;
    }
    rods[j + 1] = r;
  }
  /* bring rod (0,0) to the front by a swap */
  for (int i = 0; i < nrods; ++i) {
    if (rods[i].h == 0 && rods[i].k == 0) {
      qbo_rod t = rods[0];
      rods[0] = rods[i];
      rods[i] = t;
      break;
    }
  }
  /* good FFT sizes (Basis.cc:560-573) */
  int np[3], mx[3] = {hmax, kmax, lmax};
  for (int i = 0; i < 3; ++i) {
    int n = 2 * mx[i] + 2;
    while (!qbo_factorizable(n)) n += 2;
    np[i] = n;
  }
  if (info) {
    info[0] = size;
    info[1] = nrods;
    info[2] = np[0];
    info[3] = np[1];
    info[4] = np[2];
    info[5] = hmin_used;
    info[6] = kmin_used;
    info[7] = lmin_used;
    info[8] = hmax_used;
    info[9] = kmax_used;
    info[10] = lmax_used;
    info[11] = 0;
  }
  *rods_out = rods;
  return nrods;
}

int qbo_basis_dims(const double* a, double ecut, int* info) {
  qbo_rod* rods = 0;
  qbo_build_rods(a, ecut, &rods, info);
  free(rods);
  return info[0];
}

void qbo_basis_fill(const double* a, double ecut, int* rod_h, int* rod_k,
                    int* rod_lmin, int* rod_size, int* idx, double* kpg2,
                    double* kpgx) {
  int info[12];
  qbo_rod* rods = 0;
  const int nrods = qbo_build_rods(a, ecut, &rods, info);
  const int ng = info[0];
  double b[9];
  qbo_cell_b(a, b);
  int i = 0;
  for (int r = 0; r < nrods; ++r) {
    if (rod_h) rod_h[r] = rods[r].h;
    if (rod_k) rod_k[r] = rods[r].k;
    if (rod_lmin) rod_lmin[r] = rods[r].lmin;
    if (rod_size) rod_size[r] = rods[r].size;
    for (int l = 0; l < rods[r].size; ++l, ++i) {
      const int ih = rods[r].h, ik = rods[r].k, il = rods[r].lmin + l;
      if (idx) {
        idx[3 * i] = ih;
        idx[3 * i + 1] = ik;
        idx[3 * i + 2] = il;
      }
      /* Basis::update_g (Basis.cc:700-735), k-point 0 */
      double v[3];
      for (int j = 0; j < 3; ++j)
        v[j] = (b[j] * (0.0 + ih) + b[3 + j] * (0.0 + ik)) + b[6 + j] * (0.0 + il);
      if (kpgx) {
        kpgx[i] = v[0];
        kpgx[ng + i] = v[1];
        kpgx[2 * ng + i] = v[2];
      }
      if (kpg2) kpg2[i] = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
  }
  free(rods);
}

/* ------------------------------------------------------------------------ */
/* 1D transforms: cfftm / cfft / fftstp (FourierTransform.cc:1807-1953),     */
/* de Boor's "FFT as nested multiplication" mixed-radix scheme.              */
/* ------------------------------------------------------------------------ */
static void qbo_fftstp(int idir, const double* zin, int after, int now,
                       int before, double* zout) {
  const double twopi = 2 * 3.141592653589793;
  const double angle = twopi / (now * after);
  const double om_re = cos(angle), om_im = (double)(-idir) * sin(angle);
  double arg_re = 1.0, arg_im = 0.0;
  for (int j = 0; j < now; ++j) {
    for (int ia = 0; ia < after; ++ia) {
      for (int ib = 0; ib < before; ++ib) {
        int k = ia + ib * after + (now - 1) * before * after;
        double v_re = zin[2 * k], v_im = zin[2 * k + 1];
        for (int in = now - 2; in >= 0; --in) {
          const int l = ia + ib * after + in * before * after;
          const double t_re = v_re * arg_re - v_im * arg_im;
          const double t_im = v_re * arg_im + v_im * arg_re;
          v_re = t_re + zin[2 * l];
          v_im = t_im + zin[2 * l + 1];
        }
        const int o = ia + j * after + ib * now * after;
        zout[2 * o] = v_re;
        zout[2 * o + 1] = v_im;
      }
      const double n_re = arg_re * om_re - arg_im * om_im;
      const double n_im = arg_re * om_im + arg_im * om_re;
      arg_re = n_re;
      arg_im = n_im;
    }
  }
}

static void qbo_cfft(int idir, double* z1, double* z2, int n, int* inzee) {
  static const int prime[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  int before = n, after = 1, next = 0, now;
  do {
    const int np = prime[next];
    if ((before / np) * np < before) {
      if (++next < 12) continue;
      now = before;
      before = 1;
    } else {
      now = np;
      before /= np;
    }
    if (*inzee == 1)
      qbo_fftstp(idir, z1, after, now, before, z2);
    else
      qbo_fftstp(idir, z2, after, now, before, z1);
    *inzee = 3 - *inzee;
    after *= now;
  } while (before > 1);
}

void qbo_cfftm(double* ain, double* aout, double scale, int ntrans,
               int length, int ainc, int ajmp, int idir) {
  double* tmpa = (double*)malloc(sizeof(double) * 4 * (size_t)length);
  double* tmpb = tmpa + 2 * length;
  for (int it = 0; it < ntrans; ++it) {
    const long ibase = (long)it * ajmp;
    for (int i = 0; i < length; ++i) {
      tmpa[2 * i] = ain[2 * (ibase + (long)i * ainc)];
      tmpa[2 * i + 1] = ain[2 * (ibase + (long)i * ainc) + 1];
    }
    int inzee = 1;
    qbo_cfft(idir, tmpa, tmpb, length, &inzee);
    const double* src = inzee == 1 ? tmpa : tmpb;
    for (int i = 0; i < length; ++i) {
      aout[2 * (ibase + (long)i * ainc)] = src[2 * i] * scale;
      aout[2 * (ibase + (long)i * ainc) + 1] = src[2 * i + 1] * scale;
    }
  }
  free(tmpa);
}

/* ------------------------------------------------------------------------ */
/* FourierTransform, complex basis, one process                              */
/* ------------------------------------------------------------------------ */
struct qbo_ft {
  int ngw, nrods, np0, np1, np2, ntrans0;
  int* ifftp;   /* G -> zvec slot (FourierTransform.cc:434-455) */
  int* iunpack; /* zvec slot -> grid index (FourierTransform.cc:476-510) */
};

qbo_ft* qbo_ft_create(int ngw, int nrods, const int* rod_h, const int* rod_k,
                      const int* rod_lmin, const int* rod_size, int np0,
                      int np1, int np2, int ntrans0) {
  qbo_ft* ft = (qbo_ft*)calloc(1, sizeof(qbo_ft));
  ft->ngw = ngw;
  ft->nrods = nrods;
  ft->np0 = np0;
  ft->np1 = np1;
  ft->np2 = np2;
  ft->ntrans0 = ntrans0;
  ft->ifftp = (int*)malloc(sizeof(int) * (size_t)(ngw > 0 ? ngw : 1));
  ft->iunpack = (int*)malloc(sizeof(int) * (size_t)nrods * np2 + 1);
  int ig = 0;
  for (int r = 0; r < nrods; ++r) {
    for (int i = 0; i < rod_size[r]; ++i, ++ig) {
      int iz = i + rod_lmin[r];
      if (iz < 0) iz += np2;
      ft->ifftp[ig] = r * np2 + iz;
    }
    int h = rod_h[r], k = rod_k[r];
    if (h < 0) h += np0;
    if (k < 0) k += np1;
    for (int l = 0; l < np2; ++l)
      ft->iunpack[r * np2 + l] = h + np0 * (k + np1 * l);
  }
  return ft;
}

void qbo_ft_destroy(qbo_ft* ft) {
  if (!ft) return;
  free(ft->ifftp);
  free(ft->iunpack);
  free(ft);
}

/* backward (FourierTransform.cc:529-536, 584-980 FFT_NOLIB path):
 * f(r) = sum_G c(G) exp(+i G.r), no scaling. */
void qbo_ft_backward(const qbo_ft* ft, const double* c, double* f) {
  const int np0 = ft->np0, np1 = ft->np1, np2 = ft->np2;
  const long nz = (long)ft->nrods * np2;
  double* zvec = (double*)calloc((size_t)(2 * nz + 2), sizeof(double));
  for (int ig = 0; ig < ft->ngw; ++ig) {
    zvec[2 * ft->ifftp[ig]] = c[2 * ig];
    zvec[2 * ft->ifftp[ig] + 1] = c[2 * ig + 1];
  }
  qbo_cfftm(zvec, zvec, 1.0, ft->nrods, np2, 1, np2, -1);
  const long n012 = (long)np0 * np1 * np2;
  memset(f, 0, sizeof(double) * 2 * (size_t)n012);
  for (long i = 0; i < nz; ++i) {
    f[2 * (long)ft->iunpack[i]] = zvec[2 * i];
    f[2 * (long)ft->iunpack[i] + 1] = zvec[2 * i + 1];
  }
  free(zvec);
  const int ntrans = ft->ntrans0;
  for (int k = 0; k < np2; ++k) {
    long istart = (long)k * np0 * np1;
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, ntrans, np0, 1, np0, -1);
    istart = (long)np0 * ((np1 - ntrans) + (long)k * np1);
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, ntrans, np0, 1, np0, -1);
    istart = (long)k * np0 * np1;
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, np0, np1, np0, 1, -1);
  }
}

/* forward (FourierTransform.cc:542-553, 983-1360 FFT_NOLIB path):
 * c(G) = (1/N) sum_r f(r) exp(-i G.r); f is overwritten. */
void qbo_ft_forward(const qbo_ft* ft, double* f, double* c) {
  const int np0 = ft->np0, np1 = ft->np1, np2 = ft->np2;
  const int ntrans = ft->ntrans0;
  for (int k = 0; k < np2; ++k) {
    long istart = (long)k * np0 * np1;
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, np0, np1, np0, 1, 1);
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, ntrans, np0, 1, np0, 1);
    istart = (long)np0 * ((np1 - ntrans) + (long)k * np1);
    qbo_cfftm(f + 2 * istart, f + 2 * istart, 1.0, ntrans, np0, 1, np0, 1);
  }
  const long nz = (long)ft->nrods * np2;
  double* zvec = (double*)malloc(sizeof(double) * (size_t)(2 * nz + 2));
  for (long i = 0; i < nz; ++i) {
    zvec[2 * i] = f[2 * (long)ft->iunpack[i]];
    zvec[2 * i + 1] = f[2 * (long)ft->iunpack[i] + 1];
  }
  const double scale = 1.0 / (np0 * np1 * np2);
  qbo_cfftm(zvec, zvec, scale, ft->nrods, np2, 1, np2, 1);
  for (int ig = 0; ig < ft->ngw; ++ig) {
    c[2 * ig] = zvec[2 * ft->ifftp[ig]];
    c[2 * ig + 1] = zvec[2 * ft->ifftp[ig] + 1];
  }
  free(zvec);
}

/* ------------------------------------------------------------------------ */
/* Hamiltonian context                                                       */
/* ------------------------------------------------------------------------ */
typedef struct {
  int na, lmax, npr;
  double rc, wt[3];
  double* tau;   /* 3*na */
  int* lproj;    /* npr: l of projector ipr (NonLocalPotential::lproj) */
  double* wtp;   /* npr: weight of projector ipr (NonLocalPotential::wt) */
  double* twnl;  /* npr*ngw: after set_A (synthetic) or as given (tables) */
  int tables;    /* twnl given by the caller: set_A does not rebuild it */
} qbo_species;

struct qbo_ham {
  const qbo_ft* ft;
  int ngw;
  double omega;
  double* kpgx;  /* 3*ngw, k+G */
  double* kpgxA; /* 3*ngw, k+G-A */
  double* kpg2A; /* ngw, |k+G-A|^2 */
  double* v_r;
  double A[3];
  int nsp;
  qbo_species* sp;
};

qbo_ham* qbo_ham_create(const qbo_ft* ft, int ngw, const double* kpgx,
                        double omega, const double* v_r, int nsp,
                        const int* na, const int* lmax, const double* rc,
                        const double* wt, const double* tau) {
  qbo_ham* h = (qbo_ham*)calloc(1, sizeof(qbo_ham));
  h->ft = ft;
  h->ngw = ngw;
  h->omega = omega;
  h->kpgx = (double*)malloc(sizeof(double) * 3 * (size_t)ngw);
  memcpy(h->kpgx, kpgx, sizeof(double) * 3 * (size_t)ngw);
  h->kpgxA = (double*)malloc(sizeof(double) * 3 * (size_t)ngw);
  h->kpg2A = (double*)malloc(sizeof(double) * (size_t)ngw);
  const long n012 = (long)ft->np0 * ft->np1 * ft->np2;
  h->v_r = (double*)malloc(sizeof(double) * (size_t)n012);
  memcpy(h->v_r, v_r, sizeof(double) * (size_t)n012);
  h->nsp = nsp;
  h->sp = (qbo_species*)calloc((size_t)(nsp > 0 ? nsp : 1), sizeof(qbo_species));
  int atom0 = 0;
  for (int s = 0; s < nsp; ++s) {
    qbo_species* p = &h->sp[s];
    p->na = na[s];
    p->lmax = lmax[s];
    p->rc = rc[s];
    p->npr = 0;
    /* NonLocalPotential::init (NonLocalPotential.cc:205-250): projectors
     * ordered by l, then m; one KB channel per l */
    p->lproj = (int*)calloc(9, sizeof(int));
    p->wtp = (double*)calloc(9, sizeof(double));
    for (int l = 0; l <= p->lmax; ++l) {
      p->wt[l] = wt[3 * s + l];
      for (int m = 0; m < 2 * l + 1; ++m) {
        p->wtp[p->npr] = p->wt[l];
        p->lproj[p->npr++] = l;
      }
    }
    p->tau = (double*)malloc(sizeof(double) * 3 * (size_t)(p->na > 0 ? p->na : 1));
    memcpy(p->tau, tau + 3 * atom0, sizeof(double) * 3 * (size_t)p->na);
    atom0 += p->na;
    p->twnl = (double*)calloc((size_t)p->npr * ngw + 1, sizeof(double));
  }
  const double zero[3] = {0.0, 0.0, 0.0};
  qbo_ham_set_A(h, zero);
  return h;
}

void qbo_ham_destroy(qbo_ham* h) {
  if (!h) return;
  for (int s = 0; s < h->nsp; ++s) {
    free(h->sp[s].tau);
    free(h->sp[s].twnl);
    free(h->sp[s].lproj);
    free(h->sp[s].wtp);
  }
  free(h->sp);
  free(h->kpgx);
  free(h->kpgxA);
  free(h->kpg2A);
  free(h->v_r);
  free(h);
}

int qbo_ham_nproj(const qbo_ham* h) {
  int n = 0;
  for (int s = 0; s < h->nsp; ++s) n += h->sp[s].npr * h->sp[s].na;
  return n;
}

/* synthetic KB radial factor v_l(g) = g^l exp(-g^2 rc^2 / 2), standing in
 * for Species::dvnlg (Species.cc:1492) */
static double qbo_vnl(int l, double rc, double g) {
  const double e = exp(-0.5 * g * g * rc * rc);
  if (l == 0) return e;
  if (l == 1) return g * e;
  return g * g * e;
}

void qbo_ham_set_A(qbo_ham* h, const double* A) {
  const int ng = h->ngw;
  h->A[0] = A[0];
  h->A[1] = A[1];
  h->A[2] = A[2];
  const double value2 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
  for (int ig = 0; ig < ng; ++ig) {
    const double kx = h->kpgx[ig], ky = h->kpgx[ng + ig], kz = h->kpgx[2 * ng + ig];
    const double kpg2 = kx * kx + ky * ky + kz * kz;
    /* VectorPotential::get_kpgpa2 (VectorPotential.h:84-95) */
    double t = kpg2 + value2;
    t -= 2 * A[0] * kx;
    t -= 2 * A[1] * ky;
    t -= 2 * A[2] * kz;
    h->kpg2A[ig] = t;
    /* get_kpgpax (VectorPotential.h:110-125) */
    h->kpgxA[ig] = kx - A[0];
    h->kpgxA[ng + ig] = ky - A[1];
    h->kpgxA[2 * ng + ig] = kz - A[2];
  }
  /* update_twnl, KB branch (NonLocalPotential.cc:306-340,417-480,627-760) */
  const double pi = M_PI, fpi = 4.0 * pi;
  const double s14pi = sqrt(1.0 / fpi), s34pi = sqrt(3.0 / fpi);
  const double s54pi = sqrt(5.0 / fpi), s3 = sqrt(3.0);
  for (int s = 0; s < h->nsp; ++s) {
    qbo_species* p = &h->sp[s];
    if (p->tables) continue;
    for (int ig = 0; ig < ng; ++ig) {
      const double kpg2 = h->kpg2A[ig];
      const double tg = sqrt(kpg2);
      const double tgi = kpg2 > 0.0 ? 1.0 / sqrt(kpg2) : 0.0;
      const double tgx = h->kpgxA[ig], tgy = h->kpgxA[ng + ig], tgz = h->kpgxA[2 * ng + ig];
      int ipr = 0;
      for (int l = 0; l <= p->lmax; ++l) {
        const double v = qbo_vnl(l, p->rc, tg);
        if (l == 0) {
          p->twnl[(size_t)ng * ipr++ + ig] = s14pi * v;
        } else if (l == 1) {
          const double y1 = s34pi * tgx * tgi;
          const double y2 = s34pi * tgy * tgi;
          const double y3 = s34pi * tgz * tgi;
          p->twnl[(size_t)ng * ipr++ + ig] = y1 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y2 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y3 * v;
        } else {
          const double tgi2 = tgi * tgi;
          const double tgxx = tgx * tgx * tgi2;
          const double tgyy = tgy * tgy * tgi2;
          const double tgzz = tgz * tgz * tgi2;
          const double tgxy = tgx * tgy * tgi2;
          const double tgyz = tgy * tgz * tgi2;
          const double tgxz = tgx * tgz * tgi2;
          const double y4 = s54pi * 0.5 * (3.0 * tgzz - 1.0);
          const double y5 = s54pi * 0.5 * s3 * (tgxx - tgyy);
          const double y6 = s54pi * s3 * tgxy;
          const double y7 = s54pi * s3 * tgyz;
          const double y8 = s54pi * s3 * tgxz;
          p->twnl[(size_t)ng * ipr++ + ig] = y4 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y5 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y6 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y7 * v;
          p->twnl[(size_t)ng * ipr++ + ig] = y8 * v;
        }
      }
    }
  }
}

void qbo_ham_projector(const qbo_ham* h, int p, double* twnl, int* l,
                       double* wt, double* tau3) {
  /* flattened projector index: species, then atom block order of the
   * reference (ipr major within the species, atom minor) */
  for (int s = 0; s < h->nsp; ++s) {
    const qbo_species* sp = &h->sp[s];
    const int n = sp->npr * sp->na;
    if (p < n) {
      const int ipr = p / sp->na, ia = p % sp->na;
      if (twnl) memcpy(twnl, sp->twnl + (size_t)h->ngw * ipr, sizeof(double) * (size_t)h->ngw);
      if (l) *l = sp->lproj[ipr];
      if (wt) *wt = sp->wtp[ipr];
      if (tau3) {
        tau3[0] = sp->tau[3 * ia];
        tau3[1] = sp->tau[3 * ia + 1];
        tau3[2] = sp->tau[3 * ia + 2];
      }
      return;
    }
    p -= n;
  }
}

/* Projector tables of species s given by the caller, as NonLocalPotential::
 * init / update_twnl hold them (NonLocalPotential.cc:205-250, 261-760):
 * npr projectors with l = lproj[ipr] (0..3), weights wt[ipr] (Species::wsg),
 * twnl[ipr*ngw + ig] evaluated at |k+G-A| for the A in force.  set_A then
 * only moves the structure-factor phases. */
void qbo_ham_set_species_tables(qbo_ham* h, int s, int npr, const int* lproj,
                                const double* wt, const double* twnl) {
  qbo_species* p = &h->sp[s];
  free(p->lproj);
  free(p->wtp);
  free(p->twnl);
  p->npr = npr;
  p->lproj = (int*)calloc((size_t)(npr > 0 ? npr : 1), sizeof(int));
  p->wtp = (double*)calloc((size_t)(npr > 0 ? npr : 1), sizeof(double));
  p->twnl = (double*)calloc((size_t)npr * h->ngw + 1, sizeof(double));
  memcpy(p->lproj, lproj, sizeof(int) * (size_t)npr);
  memcpy(p->wtp, wt, sizeof(double) * (size_t)npr);
  memcpy(p->twnl, twnl, sizeof(double) * (size_t)npr * h->ngw);
  p->tables = 1;
}

/* anl column (NonLocalPotential.cc:1962-2037): twnl * (-i)^l * exp(-i(k+G-A).tau) */
static void qbo_anl_column(const qbo_ham* h, const qbo_species* sp, int ipr,
                           int ia, double* a) {
  const int ng = h->ngw;
  const double* t = sp->twnl + (size_t)ng * ipr;
  const int l = sp->lproj[ipr];
  const double mtx = -sp->tau[3 * ia], mty = -sp->tau[3 * ia + 1], mtz = -sp->tau[3 * ia + 2];
  for (int ig = 0; ig < ng; ++ig) {
    /* kpgr = -(k+G-A).tau as computed by the reference dgemm (alpha=-1) */
    double kpgr = 0.0;
    kpgr = kpgr + mtx * h->kpgxA[ig];
    kpgr = kpgr + mty * h->kpgxA[ng + ig];
    kpgr = kpgr + mtz * h->kpgxA[2 * ng + ig];
    const double s = sin(kpgr), c = cos(kpgr);
    double re, im;
    if (l == 0) {
      re = t[ig] * c;
      im = t[ig] * s;
    } else if (l == 1) {
      re = t[ig] * s;
      im = -t[ig] * c;
    } else if (l == 2) {
      re = -t[ig] * c;
      im = -t[ig] * s;
    } else {
      re = -t[ig] * s;
      im = t[ig] * c;
    }
    a[2 * ig] = re;
    a[2 * ig + 1] = im;
  }
}

/* NonLocalPotential::energy, norm-conserving complex branch
 * (NonLocalPotential.cc:1908-2170), no forces or stress.  Atom blocks of at
 * most 128 atoms as in the reference; within a block the projector index is
 * ia + ipr*block (NonLocalPotential.cc:2000). */
double qbo_nl_apply(const qbo_ham* h, const double* c, int ld, int nst,
                    const double* occ, double* cp, int nthreads) {
  const int ng = h->ngw;
  const double omega_inv = 1.0 / h->omega;
  double enl = 0.0;
  int namax = 0;
  for (int s = 0; s < h->nsp; ++s)
    if (h->sp[s].na > namax) namax = h->sp[s].na;
  const int nbs = namax > 128 ? 128 : namax;
  if (nthreads < 1) nthreads = 1;
  for (int s = 0; s < h->nsp; ++s) {
    const qbo_species* sp = &h->sp[s];
    if (sp->npr == 0 || sp->na == 0) continue;
    const int nblocks = sp->na / nbs + (sp->na % nbs == 0 ? 0 : 1);
    for (int ib = 0; ib < nblocks; ++ib) {
      const int ia0 = ib * nbs;
      const int ia1 = (ib + 1) * nbs < sp->na ? (ib + 1) * nbs : sp->na;
      const int nblk = ia1 - ia0;
      const int nprna = nblk * sp->npr;
      double* anl = (double*)malloc(sizeof(double) * 2 * (size_t)ng * nprna);
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (int col = 0; col < nprna; ++col) {
        const int ipr = col / nblk, ia = col % nblk;
        qbo_anl_column(h, sp, ipr, ia0 + ia, anl + 2 * (size_t)ng * (ia + ipr * nblk));
      }
      double* fnl = (double*)malloc(sizeof(double) * 2 * (size_t)nprna * nst);
      /* fnl = anl^H c, reference ZGEMM('C','N') summation order */
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (int n = 0; n < nst; ++n) {
        const double* cn = c + 2 * (size_t)ld * n;
        for (int i = 0; i < nprna; ++i) {
          const double* ai = anl + 2 * (size_t)ng * i;
          double t_re = 0.0, t_im = 0.0;
          for (int ig = 0; ig < ng; ++ig) {
            const double a_re = ai[2 * ig], a_im = -ai[2 * ig + 1];
            const double b_re = cn[2 * ig], b_im = cn[2 * ig + 1];
            t_re = t_re + (a_re * b_re - a_im * b_im);
            t_im = t_im + (a_re * b_im + a_im * b_re);
          }
          fnl[2 * (i + (size_t)n * nprna)] = t_re;
          fnl[2 * (i + (size_t)n * nprna) + 1] = t_im;
        }
      }
      /* Enl and D scaling (NonLocalPotential.cc:2124-2146) */
      for (int ipr = 0; ipr < sp->npr; ++ipr) {
        const double fac = sp->wtp[ipr] * omega_inv;
        for (int n = 0; n < nst; ++n) {
          const double facn = fac * (occ ? occ[n] : 0.0);
          for (int ia = 0; ia < nblk; ++ia) {
            const size_t i = ia + (size_t)ipr * nblk + (size_t)n * nprna;
            const double t_re = fnl[2 * i], t_im = fnl[2 * i + 1];
            enl += facn * (t_re * t_re + t_im * t_im);
            fnl[2 * i] = fac * t_re;
            fnl[2 * i + 1] = fac * t_im;
          }
        }
      }
      /* cp += anl * fnl, reference ZGEMM('N','N') with beta = 1 */
      if (cp) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int n = 0; n < nst; ++n) {
          double* cpn = cp + 2 * (size_t)ld * n;
          for (int i = 0; i < nprna; ++i) {
            const double f_re = fnl[2 * (i + (size_t)n * nprna)];
            const double f_im = fnl[2 * (i + (size_t)n * nprna) + 1];
            const double* ai = anl + 2 * (size_t)ng * i;
            for (int ig = 0; ig < ng; ++ig) {
              const double a_re = ai[2 * ig], a_im = ai[2 * ig + 1];
              cpn[2 * ig] = cpn[2 * ig] + (f_re * a_re - f_im * a_im);
              cpn[2 * ig + 1] = cpn[2 * ig + 1] + (f_re * a_im + f_im * a_re);
            }
          }
        }
      }
      free(fnl);
      free(anl);
    }
  }
  return enl;
}

/* cp += 0.5 |k+G-A|^2 c  (EnergyFunctional.cc:1670-1690) */
void qbo_kinetic_add(const qbo_ham* h, const double* c, int ld, int nst,
                     double* cp) {
  for (int n = 0; n < nst; ++n) {
    const double* cn = c + 2 * (size_t)ld * n;
    double* cpn = cp + 2 * (size_t)ld * n;
    for (int ig = 0; ig < h->ngw; ++ig) {
      const double x = 0.5 * h->kpg2A[ig];
      cpn[2 * ig] = cpn[2 * ig] + x * cn[2 * ig];
      cpn[2 * ig + 1] = cpn[2 * ig + 1] + x * cn[2 * ig + 1];
    }
  }
}

/* SlaterDet::rs_mul_add complex branch (SlaterDet.cc:1025-1037) */
void qbo_rs_mul_add(const qbo_ham* h, const double* c, int ld, int nst,
                    double* cp, int nthreads) {
  const qbo_ft* ft = h->ft;
  const long n012 = (long)ft->np0 * ft->np1 * ft->np2;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
  {
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
    double* ctmp = (double*)malloc(sizeof(double) * 2 * (size_t)(h->ngw + 1));
#pragma omp for schedule(dynamic, 1)
    for (int n = 0; n < nst; ++n) {
      qbo_ft_backward(ft, c + 2 * (size_t)ld * n, tmp);
      for (long i = 0; i < n012; ++i) {
        tmp[2 * i] = tmp[2 * i] * h->v_r[i];
        tmp[2 * i + 1] = tmp[2 * i + 1] * h->v_r[i];
      }
      qbo_ft_forward(ft, tmp, ctmp);
      double* cpn = cp + 2 * (size_t)ld * n;
      for (int ig = 0; ig < h->ngw; ++ig) {
        cpn[2 * ig] = cpn[2 * ig] + ctmp[2 * ig];
        cpn[2 * ig + 1] = cpn[2 * ig + 1] + ctmp[2 * ig + 1];
      }
    }
    free(tmp);
    free(ctmp);
  }
}

/* EnergyFunctional::energy(compute_hpsi=true): clear, NL, kinetic, local */
double qbo_hpsi(const qbo_ham* h, const double* c, int ld, int nst,
                const double* occ, double* cp, int nthreads) {
  memset(cp, 0, sizeof(double) * 2 * (size_t)ld * nst);
  const double enl = qbo_nl_apply(h, c, ld, nst, occ, cp, nthreads);
  qbo_kinetic_add(h, c, ld, nst, cp);
  qbo_rs_mul_add(h, c, ld, nst, cp, nthreads);
  return enl;
}

void qbo_compute_density(const qbo_ft* ft, const double* c, int ld, int nst,
                         const double* occ, double weight, double omega,
                         double* rho, int nthreads) {
  const long n012 = (long)ft->np0 * ft->np1 * ft->np2;
  const double prefac = weight / omega;
  double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
  (void)nthreads;
  for (int n = 0; n < nst; ++n) {
    const double fac = prefac * occ[n];
    if (fac > 0.0) {
      qbo_ft_backward(ft, c + 2 * (size_t)ld * n, tmp);
      for (long i = 0; i < n012; ++i)
        rho[i] += fac * (tmp[2 * i] * tmp[2 * i] + tmp[2 * i + 1] * tmp[2 * i + 1]);
    }
  }
  free(tmp);
}

double qbo_update_density(const qbo_ft* ft, const double* c, int ld, int nst,
                          const double* occ, double omega, double* rho,
                          int nthreads) {
  const long n012 = (long)ft->np0 * ft->np1 * ft->np2;
  memset(rho, 0, sizeof(double) * (size_t)n012);
  if (nthreads > 1 && nst > 1) {
    /* states split over threads; the partial sums are added in thread
     * order, so the result differs from one thread only by rounding */
    int nt = nthreads < nst ? nthreads : nst;
    double* part = (double*)calloc((size_t)nt * n012, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int t = 0; t < nt; ++t) {
      const int n0 = (int)((long)nst * t / nt), n1 = (int)((long)nst * (t + 1) / nt);
      qbo_compute_density(ft, c + 2 * (size_t)ld * n0, ld, n1 - n0, occ + n0,
                          1.0, omega, part + (size_t)t * n012, 1);
    }
    for (int t = 0; t < nt; ++t)
      for (long i = 0; i < n012; ++i) rho[i] += part[(size_t)t * n012 + i];
    free(part);
  } else {
    qbo_compute_density(ft, c, ld, nst, occ, 1.0, omega, rho, 1);
  }
  double nel = 0.0;
  for (long i = 0; i < n012; ++i) nel += rho[i];
  nel *= omega / (double)n012;
  return nel;
}

void qbo_current_rs(const qbo_ft* ft, const double* kpgx, int ngw,
                    const double* c, int ld, int nst, const double* occ,
                    double omega, const double* A, double nel, double* J,
                    int nthreads) {
  const long n012 = (long)ft->np0 * ft->np1 * ft->np2;
  const double vol_elem = omega / (double)n012;
  const double prefac = 1.0 / omega;
  double* t1 = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
  double* t2 = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
  double* rc = (double*)malloc(sizeof(double) * 2 * (size_t)(ngw + 1));
  double* cur = (double*)malloc(sizeof(double) * (size_t)n012);
  (void)nthreads;
  for (int d = 0; d < 3; ++d) {
    memset(cur, 0, sizeof(double) * (size_t)n012);
    double* acc = (double*)calloc(2 * (size_t)n012, sizeof(double));
    for (int n = 0; n < nst; ++n) {
      const double fac = prefac * occ[n];
      if (!(fac > 0.0)) continue;
      const double* cn = c + 2 * (size_t)ld * n;
      for (int ig = 0; ig < ngw; ++ig) {
        const double k = kpgx[(size_t)d * ngw + ig];
        /* (0,1)*k*c = (-k c_im, k c_re) */
        rc[2 * ig] = -(k * cn[2 * ig + 1]);
        rc[2 * ig + 1] = k * cn[2 * ig];
      }
      qbo_ft_backward(ft, cn, t1);
      qbo_ft_backward(ft, rc, t2);
      for (long i = 0; i < n012; ++i) {
        /* fac * conj(t1) * t2 */
        const double a_re = fac * t1[2 * i], a_im = -(fac * t1[2 * i + 1]);
        const double b_re = t2[2 * i], b_im = t2[2 * i + 1];
        acc[2 * i] += a_re * b_re - a_im * b_im;
        acc[2 * i + 1] += a_re * b_im + a_im * b_re;
      }
    }
    for (long i = 0; i < n012; ++i) cur[i] += -acc[2 * i + 1];
    double tot = 0.0;
    for (long i = 0; i < n012; ++i) tot += vol_elem * cur[i];
    J[d] = tot + A[d] * nel;
    free(acc);
  }
  free(t1);
  free(t2);
  free(rc);
  free(cur);
}

void qbo_current_g(const double* kpgx, int ngw, const double* c, int ld,
                   int nst, const double* occ, const double* A, double nel,
                   double* J) {
  for (int d = 0; d < 3; ++d) {
    double tot = 0.0;
    for (int n = 0; n < nst; ++n) {
      const double* cn = c + 2 * (size_t)ld * n;
      double s = 0.0;
      for (int ig = 0; ig < ngw; ++ig)
        s += kpgx[(size_t)d * ngw + ig] * (cn[2 * ig] * cn[2 * ig] + cn[2 * ig + 1] * cn[2 * ig + 1]);
      tot += occ[n] * s;
    }
    J[d] = -tot + A[d] * nel;
  }
}

/* ExponentialWavefunctionStepper::exponential with one time step
 * (ExponentialWavefunctionStepper.cc:51-148), 4th-order Taylor series. */
static void qbo_exponential(const qbo_ham* h, double* wf, int ld, int nst,
                            const double* occ, double dt1, double* dwf,
                            double* expwf, int nthreads) {
  const size_t len = 2 * (size_t)ld * nst;
  qbo_hpsi(h, wf, ld, nst, occ, dwf, nthreads);
  memcpy(expwf, wf, sizeof(double) * len);
  double f_re = 1.0, f_im = 0.0;
  for (int N = 1; N <= 4; ++N) {
    /* factor1 *= -complex(0,1)*dt1/double(N) */
    const double m_re = -0.0 * dt1 / (double)N, m_im = -1.0 * dt1 / (double)N;
    const double n_re = f_re * m_re - f_im * m_im;
    const double n_im = f_re * m_im + f_im * m_re;
    f_re = n_re;
    f_im = n_im;
    if (N != 1) {
      memcpy(wf, dwf, sizeof(double) * len);
      qbo_hpsi(h, wf, ld, nst, occ, dwf, nthreads);
    }
    /* expwf += factor1 * dwf  (ComplexMatrix::axpy -> zaxpy) */
    for (size_t i = 0; i < len / 2; ++i) {
      const double x_re = dwf[2 * i], x_im = dwf[2 * i + 1];
      expwf[2 * i] = expwf[2 * i] + (f_re * x_re - f_im * x_im);
      expwf[2 * i + 1] = expwf[2 * i + 1] + (f_re * x_im + f_im * x_re);
    }
  }
  memcpy(wf, expwf, sizeof(double) * len);
}

double qbo_etrs_step(qbo_ham* h, double* psi, int ld, int nst,
                     const double* occ, double dt, const double* A_t,
                     const double* A_tdt, double* rho_mid, int nthreads) {
  const size_t len = 2 * (size_t)ld * nst;
  double* dwf = (double*)malloc(sizeof(double) * len);
  double* expwf = (double*)malloc(sizeof(double) * len);
  double* newwf = (double*)malloc(sizeof(double) * len);
  const double dt1 = 0.5 * dt;
  /* preupdate (ExponentialWavefunctionStepper.cc:153-205) with H(t) */
  qbo_ham_set_A(h, A_t);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  memcpy(newwf, psi, sizeof(double) * len);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  /* update (ExponentialWavefunctionStepper.cc:241-276): density of the
   * predicted psi(t+dt); the Hamiltonian moves to A(t+dt) */
  double nel = 0.0;
  if (rho_mid)
    nel = qbo_update_density(h->ft, psi, ld, nst, occ, h->omega, rho_mid, nthreads);
  qbo_ham_set_A(h, A_tdt);
  memcpy(psi, newwf, sizeof(double) * len);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  free(dwf);
  free(expwf);
  free(newwf);
  return nel;
}

/* LDA exchange + Perdew-Zunger (1981) parametrisation of the Ceperley-Alder
 * correlation energy, spin unpolarised, Hartree units -- the functional of
 * LDAFunctional::xc_unpolarized (functionals/LDAFunctional.cc:102-160).
 * rs = (3/(4 pi rho))^(1/3); exchange vx = -(3/pi)^(1/3) rho^(1/3) written
 * through rs; correlation: A ln rs + B + C rs ln rs + D rs for rs < 1,
 * gamma / (1 + beta1 sqrt(rs) + beta2 rs) otherwise, with C and D fixed by
 * continuity of e_c and v_c at rs = 1. */
void qbo_lda(double rh, double* ee, double* vv) {
  const double c1 = 0.6203504908994001;   /* (3/(4 pi))^(1/3) */
  const double c3 = -0.610887057711;      /* -(4/3)(3/(4 pi))/(4/(9 pi))^(1/3) */
  const double A = 0.0311, B = -0.048, b1 = 1.0529, b2 = 0.3334, G = -0.1423;
  const double D = G / (1.0 + b1 + b2) - B;
  const double C = -A - D - G * ((b1 / 2.0 + b2) / ((1.0 + b1 + b2) * (1.0 + b1 + b2)));
  *ee = 0.0;
  *vv = 0.0;
  if (rh > 0.0) {
    const double ro13 = cbrt(rh);
    const double rs = c1 / ro13;
    const double vx = c3 / rs, ex = 0.75 * vx;
    double ec, vc;
    if (rs < 1.0) {
      const double logrs = log(rs);
      ec = A * logrs + B + C * rs * logrs + D * rs;
      vc = A * logrs + (B - A / 3.0) + (2.0 / 3.0) * C * rs * logrs + ((2.0 * D - C) / 3.0) * rs;
    } else {
      const double sqrtrs = sqrt(rs);
      const double den = 1.0 + b1 * sqrtrs + b2 * rs;
      ec = G / den;
      vc = ec * (1.0 + (7.0 / 6.0) * b1 * sqrtrs + (4.0 / 3.0) * b2 * rs) / den;
    }
    *ee = ex + ec;
    *vv = vx + vc;
  }
}

void qbo_density_g(const qbo_ft* vft, const double* rho, double omega, double* rhog) {
  const long n012 = (long)vft->np0 * vft->np1 * vft->np2;
  double* f = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
  for (long i = 0; i < n012; ++i) {
    f[2 * i] = omega * rho[i];
    f[2 * i + 1] = 0.0;
  }
  qbo_ft_forward(vft, f, rhog);
  free(f);
}

double qbo_update_vhxc(const qbo_ft* vft, const double* g2, int ngv,
                       const double* vion_g, const double* rhopst_g,
                       const double* rho, double omega, double* v_r, double* en) {
  const long n012 = (long)vft->np0 * vft->np1 * vft->np2;
  double* f = (double*)malloc(sizeof(double) * 2 * (size_t)n012);
  double* rg = (double*)malloc(sizeof(double) * 2 * (size_t)(ngv + 1));
  qbo_density_g(vft, rho, omega, rg);
  const double omega_inv = 1.0 / omega, fpi = 4.0 * M_PI;
  double ehsum = 0.0, eps = 0.0;
  for (int ig = 0; ig < ngv; ++ig) {
    /* g2i = (1/|G|)^2 (Basis.cc:730-739) */
    const double g = sqrt(g2[ig]);
    const double gi = g > 0.0 ? 1.0 / g : 0.0;
    const double g2i = gi * gi;
    const double re = omega_inv * rg[2 * ig], im = omega_inv * rg[2 * ig + 1];
    /* eps: ddot of rhoelg with vion_local_g (EnergyFunctional.cc:456-469) */
    eps += re * vion_g[2 * ig] + im * vion_g[2 * ig + 1];
    const double tr = re + (rhopst_g ? rhopst_g[2 * ig] : 0.0);
    const double ti = im + (rhopst_g ? rhopst_g[2 * ig + 1] : 0.0);
    ehsum += (tr * tr + ti * ti) * g2i;
    /* vlocal_g = vion_local_g + 4 pi hamil_rhogt g2i (EnergyFunctional.cc:510-515) */
    rg[2 * ig] = vion_g[2 * ig] + fpi * tr * g2i;
    rg[2 * ig + 1] = vion_g[2 * ig + 1] + fpi * ti * g2i;
  }
  qbo_ft_backward(vft, rg, f);
  double exc = 0.0;
  for (long i = 0; i < n012; ++i) {
    double e, v;
    qbo_lda(rho[i], &e, &v);
    exc += rho[i] * e;
    v_r[i] = v + f[2 * i];
  }
  /* complex basis: vfact 0.5 (EnergyFunctional.cc:494-497) */
  const double ehart = 0.5 * omega * fpi * ehsum;
  if (en) {
    en[0] = ehart;
    en[1] = exc * omega / (double)n012; /* XCPotential.cc:145-190 */
    en[2] = eps * omega;
  }
  free(f);
  free(rg);
  return ehart;
}

/* AETRS, ExponentialWavefunctionStepper with approximated_ (Exponential-
 * WavefunctionStepper.cc:153-276, SelfConsistentPotential.cc:46-73) on top of
 * the self-consistent loop top (vft != NULL) or a fixed potential (vft ==
 * NULL): vhist [3][n012] holds v_r of the last three steps, *stored counts
 * them.  From the third stored step on the step is two half-step
 * exponentials, the second with v = 3 v2 - 3 v1 + 1 v0 and A_t; before that
 * it is the ETRS step.  The predicted state the reference also computes in
 * that case is overwritten there unused (:218-225), so it is not formed
 * here. */
double qbo_aetrs_step(qbo_ham* h, double* psi, int ld, int nst, const double* occ,
                      double dt, const double* A_t, const double* A_tdt,
                      const qbo_ft* vft, const double* g2, int ngv,
                      const double* vion_g, const double* rhopst_g, double* vhist,
                      int* stored, int nthreads) {
  const long n012 = (long)h->ft->np0 * h->ft->np1 * h->ft->np2;
  const size_t len = 2 * (size_t)ld * nst;
  double* rho = (double*)malloc(sizeof(double) * (size_t)n012);
  double* dwf = (double*)malloc(sizeof(double) * len);
  double* expwf = (double*)malloc(sizeof(double) * len);
  double* newwf = (double*)malloc(sizeof(double) * len);
  const double dt1 = 0.5 * dt;
  if (vft) {
    qbo_update_density(h->ft, psi, ld, nst, occ, h->omega, rho, nthreads);
    qbo_update_vhxc(vft, g2, ngv, vion_g, rhopst_g, rho, h->omega, h->v_r, NULL);
  }
  /* potential_[0] = potential_[1]; [1] = [2]; [2] = current */
  memcpy(vhist, vhist + n012, sizeof(double) * (size_t)n012);
  memcpy(vhist + n012, vhist + 2 * n012, sizeof(double) * (size_t)n012);
  memcpy(vhist + 2 * n012, h->v_r, sizeof(double) * (size_t)n012);
  if (*stored < 3) ++*stored;
  qbo_ham_set_A(h, A_t);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  double nel = 0.0;
  if (*stored >= 3) {
    for (long i = 0; i < n012; ++i)
      h->v_r[i] = 3.0 * vhist[2 * n012 + i] - 3.0 * vhist[n012 + i] + 1.0 * vhist[i];
    qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
    qbo_ham_set_A(h, A_tdt);
  } else {
    memcpy(newwf, psi, sizeof(double) * len);
    qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
    nel = qbo_update_density(h->ft, psi, ld, nst, occ, h->omega, rho, nthreads);
    if (vft) qbo_update_vhxc(vft, g2, ngv, vion_g, rhopst_g, rho, h->omega, h->v_r, NULL);
    qbo_ham_set_A(h, A_tdt);
    memcpy(psi, newwf, sizeof(double) * len);
    qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  }
  free(rho);
  free(dwf);
  free(expwf);
  free(newwf);
  return nel;
}

double qbo_etrs_step_hxc(qbo_ham* h, double* psi, int ld, int nst,
                         const double* occ, double dt, const double* A_t,
                         const double* A_tdt, const qbo_ft* vft,
                         const double* g2, int ngv, const double* vion_g,
                         const double* rhopst_g, double* rho_mid, int nthreads) {
  const long n012 = (long)h->ft->np0 * h->ft->np1 * h->ft->np2;
  const size_t len = 2 * (size_t)ld * nst;
  double* rho = (double*)malloc(sizeof(double) * (size_t)n012);
  double* dwf = (double*)malloc(sizeof(double) * len);
  double* expwf = (double*)malloc(sizeof(double) * len);
  double* newwf = (double*)malloc(sizeof(double) * len);
  const double dt1 = 0.5 * dt;
  /* loop top: density of psi(t) and the Hamiltonian built from it */
  qbo_update_density(h->ft, psi, ld, nst, occ, h->omega, rho, nthreads);
  qbo_update_vhxc(vft, g2, ngv, vion_g, rhopst_g, rho, h->omega, h->v_r, NULL);
  qbo_ham_set_A(h, A_t);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  memcpy(newwf, psi, sizeof(double) * len);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  const double nel = qbo_update_density(h->ft, psi, ld, nst, occ, h->omega, rho, nthreads);
  if (rho_mid) memcpy(rho_mid, rho, sizeof(double) * (size_t)n012);
  qbo_update_vhxc(vft, g2, ngv, vion_g, rhopst_g, rho, h->omega, h->v_r, NULL);
  qbo_ham_set_A(h, A_tdt);
  memcpy(psi, newwf, sizeof(double) * len);
  qbo_exponential(h, psi, ld, nst, occ, dt1, dwf, expwf, nthreads);
  free(rho);
  free(dwf);
  free(expwf);
  free(newwf);
  return nel;
}

void qbo_ham_get_vr(const qbo_ham* h, double* v) {
  const long n012 = (long)h->ft->np0 * h->ft->np1 * h->ft->np2;
  memcpy(v, h->v_r, sizeof(double) * (size_t)n012);
}
