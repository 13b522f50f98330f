/* Single-rank build configuration used only to compile the reference's own
 * Basis/FourierTransform/UnitCell sources into oracle/_ref (test
 * infrastructure; never part of the product).  USE_MPI is left undefined so
 * the sources take their serial branches; the two MPI queries that the
 * FourierTransform constructor makes unconditionally are answered by
 * ref_context_stub.cc with a one-process communicator. */
#ifndef QBG_REF_STUB_CONFIG_H
#define QBG_REF_STUB_CONFIG_H
#define FC_FUNC(name, NAME) name##_
#define FFT_NOLIB 1
int MPI_Comm_size(int comm, int* size);
int MPI_Comm_rank(int comm, int* rank);
/* Species.cc aborts through MPI on a bad Hubbard input (never reached here) */
#define MPI_COMM_WORLD 0
int MPI_Abort(int comm, int code);
#endif
