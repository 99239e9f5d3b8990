/* Minimal stand-in for <mpi.h> so the reference corr_pc sources compile
 * without an MPI installation.  The reference only calls MPI::Init,
 * MPI::Finalize and COMM_WORLD.Get_rank/Get_size (main.cpp:31,59,78;
 * do_corr.cpp:26-27) and never uses the values to split work, so a
 * single-rank stub reproduces its behaviour exactly.
 * Test infrastructure only: never linked into the product library. */
#ifndef CPC_ORACLE_MPI_STUB_H
#define CPC_ORACLE_MPI_STUB_H
namespace MPI {
struct Comm_stub {
  int Get_rank() const { return 0; }
  int Get_size() const { return 1; }
};
static Comm_stub COMM_WORLD;
inline void Init(int &, char **&) {}
inline void Finalize() {}
}  // namespace MPI
#endif
