// unreached.cpp -- link-time stand-ins for the reference functions that
// Particles.cxx and Domain.cxx reference but the sub-cycle oracle
// (sub_driver.cpp) never calls: the Barnes-Hut tree (HACC without -R/-O), the
// restart I/O (MPI-IO) and the MPI Cartesian decomposition queries
// (Domain::initialize).  Each aborts if it is ever reached.
//
// TEST INFRASTRUCTURE ONLY (the oracle's recipe in oracle/Makefile).
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "BHForceTree.h"
#include "Partition.h"
#include "RestartIO.h"

namespace {
[[noreturn]] void unreached(const char *what) {
  fprintf(stderr, "sub_driver: %s is outside the sub-cycle oracle\n", what);
  abort();
}
}  // namespace

BHForceTree::BHForceTree(POSVEL_T *, POSVEL_T *, ID_T, POSVEL_T *, POSVEL_T *, POSVEL_T *,
                         POSVEL_T *, POSVEL_T *, POSVEL_T *, POSVEL_T *, POSVEL_T, ForceLaw *,
                         float) {
  unreached("BHForceTree");
}
BHForceTree::~BHForceTree() {}
void BHForceTree::treeForceGadgetTopDown(ID_T, POSVEL_T, POSVEL_T) {
  unreached("BHForceTree::treeForceGadgetTopDown");
}
void BHForceTree::treeForceGadgetTopDownFast2(ID_T, POSVEL_T, POSVEL_T, vector<POSVEL_T> *,
                                              vector<POSVEL_T> *, vector<POSVEL_T> *,
                                              vector<POSVEL_T> *, double *, double *) {
  unreached("BHForceTree::treeForceGadgetTopDownFast2");
}
RestartIO::RestartIO(int, char *, MPI_Comm) { unreached("RestartIO"); }
void RestartIO::WriteRestart(int &, float *, float *, float *, float *, float *, float *, float *,
                             int64_t *, uint16_t *) {
  unreached("RestartIO::WriteRestart");
}
int RestartIO::ReadRestart(float *&, float *&, float *&, float *&, float *&, float *&, float *&,
                           int64_t *&, uint16_t *&) {
  unreached("RestartIO::ReadRestart");
}
void Partition::getDecompSize(int[]) { unreached("Partition::getDecompSize"); }
void Partition::getMyPosition(int[]) { unreached("Partition::getMyPosition"); }
