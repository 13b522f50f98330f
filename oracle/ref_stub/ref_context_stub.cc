// One-process stand-in for the reference's BLACS/MPI Context and for the two
// MPI queries made by its FourierTransform constructor.  It is test
// infrastructure: it exists only so that the reference's own serial
// Basis/FourierTransform/UnitCell sources can be compiled into oracle/_ref and
// used as the pinned FFT oracle.  Every member answers as rank 0 of a 1x1 grid.
#include <config.h>
#include "Context.h"
#include <cstdlib>

int MPI_Comm_size(int, int* size) { *size = 1; return 0; }
int MPI_Comm_rank(int, int* rank) { *rank = 0; return 0; }
int MPI_Abort(int, int code) { std::abort(); return code; }

Context::Context() : pimpl_(0) {}
Context::~Context() {}
int Context::ictxt() const { return 0; }
int Context::myrow() const { return 0; }
int Context::mycol() const { return 0; }
int Context::nprow() const { return 1; }
int Context::npcol() const { return 1; }
int Context::size() const { return 1; }
int Context::myproc() const { return 0; }
int Context::mype() const { return 0; }
bool Context::onpe0() const { return true; }
bool Context::oncoutpe() const { return true; }
int Context::coutpe() const { return 0; }
bool Context::active() const { return true; }
void Context::barrier() const {}
MPI_Comm Context::comm() const { return 0; }
void Context::isend(int, int, int*, int, int, int) const {}
void Context::irecv(int, int, int*, int, int, int) const {}
void Context::dsend(int, int, double*, int, int, int) const {}
void Context::drecv(int, int, double*, int, int, int) const {}
// broadcasts from the only process are no-ops (used by SpeciesReader)
int Context::pmap(int, int) const { return 0; }
void Context::dbcast_send(int, int, double*, int) const {}
void Context::dbcast_recv(int, int, double*, int, int, int) const {}
void Context::ibcast_send(int, int, int*, int) const {}
void Context::ibcast_recv(int, int, int*, int, int, int) const {}
void Context::string_bcast(std::string&, int) const {}
