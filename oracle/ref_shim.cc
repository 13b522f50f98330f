// C entry points over the reference's own Basis and FourierTransform classes.
// Compiled together with those unmodified reference sources (read in place,
// never copied) into oracle/_ref/libqbref.so by oracle/build_ref.sh.  This is
// test infrastructure: the golden-fixture generator and the CPU tests call it
// to pin the oracle restatement in oracle/qbo.c; nothing in the product links it.
#include <config.h>
#include "Basis.h"
#include "FourierTransform.h"
#include "UnitCell.h"
#include "LDAFunctional.h"
#include "Species.h"
#include "SpeciesReader.h"
#include <complex>
#include <vector>

namespace {
struct RefBasis {
  Context ctxt;
  Basis* basis;
};
}

extern "C" {

// a: 9 doubles, cell vectors a0,a1,a2 (bohr); ecut in Hartree as Basis::resize
// expects; force_complex=1 gives the full-sphere basis used by TDDFT.
void* qbref_basis_create(const double* a, double ecut, int force_complex) {
  RefBasis* rb = new RefBasis;
  rb->basis = new Basis(rb->ctxt, D3vector(0.0, 0.0, 0.0), force_complex != 0);
  UnitCell cell(D3vector(a[0], a[1], a[2]), D3vector(a[3], a[4], a[5]),
                D3vector(a[6], a[7], a[8]));
  rb->basis->resize(cell, cell, ecut);
  return rb;
}

void qbref_basis_destroy(void* h) {
  RefBasis* rb = static_cast<RefBasis*>(h);
  delete rb->basis;
  delete rb;
}

// info[0]=size, [1]=nrods, [2..4]=np, [5..7]=idxmin, [8..10]=idxmax, [11]=real
void qbref_basis_info(void* h, int* info) {
  const Basis& b = *static_cast<RefBasis*>(h)->basis;
  info[0] = b.size();
  info[1] = b.nrods();
  for (int i = 0; i < 3; ++i) {
    info[2 + i] = b.np(i);
    info[5 + i] = b.idxmin(i);
    info[8 + i] = b.idxmax(i);
  }
  info[11] = b.real() ? 1 : 0;
}

void qbref_basis_rods(void* h, int* rh, int* rk, int* rlmin, int* rsize) {
  const Basis& b = *static_cast<RefBasis*>(h)->basis;
  for (int i = 0; i < b.nrod_loc(); ++i) {
    rh[i] = b.rod_h(i);
    rk[i] = b.rod_k(i);
    rlmin[i] = b.rod_lmin(i);
    rsize[i] = b.rod_size(i);
  }
}

// idx[3*ng], kpg2[ng], kpgx[3*ng] (x block, y block, z block)
void qbref_basis_tables(void* h, int* idx, double* kpg2, double* kpgx) {
  const Basis& b = *static_cast<RefBasis*>(h)->basis;
  const int ng = b.localsize();
  for (int i = 0; i < 3 * ng; ++i) idx[i] = b.idx(i);
  for (int i = 0; i < ng; ++i) kpg2[i] = b.kpg2(i);
  for (int i = 0; i < 3 * ng; ++i) kpgx[i] = b.kpgx(i);
}

void* qbref_ft_create(void* h, int np0, int np1, int np2) {
  return new FourierTransform(*static_cast<RefBasis*>(h)->basis, np0, np1, np2);
}

void qbref_ft_destroy(void* ft) { delete static_cast<FourierTransform*>(ft); }

// c: interleaved complex [ngw]; f: interleaved complex [np0*np1*np2]
void qbref_ft_backward(void* ft, const double* c, double* f) {
  static_cast<FourierTransform*>(ft)->backward(
      reinterpret_cast<const std::complex<double>*>(c),
      reinterpret_cast<std::complex<double>*>(f));
}

// f is overwritten, as in FourierTransform::forward.
void qbref_ft_forward(void* ft, double* f, double* c) {
  static_cast<FourierTransform*>(ft)->forward(
      reinterpret_cast<std::complex<double>*>(f),
      reinterpret_cast<std::complex<double>*>(c));
}

// LDAFunctional::setxc (functionals/LDAFunctional.cc:39-101), spin
// unpolarised: exc[i], vxc[i] for rho[i], i < n.
void qbref_lda(int n, const double* rho, double* exc, double* vxc) {
  std::vector<std::vector<double> > rhoe(1, std::vector<double>(rho, rho + n));
  LDAFunctional f(rhoe);
  f.setxc();
  for (int i = 0; i < n; ++i) {
    exc[i] = f.exc[i];
    vxc[i] = f.vxc1[i];
  }
}

// ---- Species (Species.cc, SpeciesReader.cc): a pseudopotential read from
// its file by the reference's own reader and initialised by
// Species::initialize (radial Bessel transforms, KB weights, splines).
namespace {
struct RefSpecies {
  Context ctxt;
  Species* sp;
};
}

// path: species file (QSO XML, UPF, ...); rcps: Gaussian pseudo-charge
// radius.  NULL when reading or initialising fails.
void* qbref_species_load(const char* path, double rcps) {
  RefSpecies* r = new RefSpecies;
  r->sp = new Species(r->ctxt, "sp");
  try {
    SpeciesReader rd(r->ctxt);
    rd.readSpecies(*r->sp, path);
    if (!r->sp->initialize(rcps)) throw 1;
  } catch (...) {
    delete r->sp;
    delete r;
    return nullptr;
  }
  return r;
}

void qbref_species_destroy(void* h) {
  RefSpecies* r = static_cast<RefSpecies*>(h);
  delete r->sp;
  delete r;
}

// info[0]=lmax [1]=llocal [2]=nchannels [3]=nlm [4]=zval [5]=nquad
// [6]=ultrasoft [7]=oncv
void qbref_species_info(void* h, int* info) {
  Species& s = *static_cast<RefSpecies*>(h)->sp;
  info[0] = s.lmax();
  info[1] = s.llocal();
  info[2] = s.nchannels();
  info[3] = s.nlm();
  info[4] = s.zval();
  info[5] = s.nquad();
  info[6] = s.ultrasoft() ? 1 : 0;
  info[7] = 0;
}

// Kleinman-Bylander weight wsg(l, ic) = 1 / <phi|dV|phi>
double qbref_species_wsg(void* h, int l, int ic) {
  return static_cast<RefSpecies*>(h)->sp->wsg(l, ic);
}

// v[i] = the radial projector of (l, ic) at |G| = g[i] (Species::dvnlg)
void qbref_species_vnlg(void* h, int l, int ic, int n, const double* g, double* v) {
  Species& s = *static_cast<RefSpecies*>(h)->sp;
  for (int i = 0; i < n; ++i) {
    double dv;
    s.dvnlg(l, ic, g[i], v[i], dv);
  }
}

}  // extern "C"
