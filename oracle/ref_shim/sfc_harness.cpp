/*
 * sfc_harness.cpp -- C entry point to the reference's Lebesgue-to-Hilbert key
 * conversion (MolecularDynamics/BarnesHutParallel/SpaceFillingCurves/src/Tree.cpp:70-104),
 * compiled from the reference's own source with the single-process mpi.h
 * stand-in.  TEST INFRASTRUCTURE ONLY.
 *
 * Keys use the reference's MD convention: 21 levels of 3 bits, level 1 in
 * bits 62..60, the child number sonNumber = [x>=mid] + 2[y>=mid] + 4[z>=mid]
 * (Tree.cpp:442).
 */
#include "Tree.h"

// Tree.h declares a one-argument form; Tree.cpp:90 defines this one (level =
// number of levels of the key that are converted).
keytype Lebesgue2Hilbert(keytype lebesgue, int level);

// globals the reference defines in its main.cpp (not compiled here)
MPI_Datatype mpiParticle = 0;
structlog LOGCFG = {};

extern "C" void ref_lebesgue2hilbert(const unsigned long *lebesgue, unsigned long *hilbert, long n, int level) {
    for (long i = 0; i < n; i++) hilbert[i] = Lebesgue2Hilbert(lebesgue[i], level);
}
