/* Single-rank stand-in for the MPI calls the reference's OpenMP drivers make
 * (rank/size queries, MPI_Abort, MPI_Bcast, the struct/op registration in the
 * chain-KMC base class). Test infrastructure only: the oracle runs one process. */
#ifndef LMC_ORACLE_SHIM_MPI_H_
#define LMC_ORACLE_SHIM_MPI_H_
#include <cstddef>
#include <cstdlib>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef std::ptrdiff_t MPI_Aint;
typedef void MPI_User_function(void *, void *, int *, MPI_Datatype *);
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 3
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_IN_PLACE nullptr
inline int MPI_Init_thread(int *, char ***, int, int *provided) { if (provided) *provided = 1; return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) { *op = 0; return 0; }
inline int MPI_Op_free(MPI_Op *) { return 0; }
inline int MPI_Type_create_struct(int, const int *, const MPI_Aint *, const MPI_Datatype *, MPI_Datatype *t) { *t = 0; return 0; }
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }
#endif
