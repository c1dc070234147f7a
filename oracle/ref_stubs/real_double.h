/*
 * Pre-included (g++ -include) when compiling the CPU reference as the FP64
 * oracle. It defines the reference's precision header guard first, so the
 * reference's own `using real = float` is skipped and `real` is double.
 */
#ifndef INCLUDE_TLBM_DEFINTIONS_H_
#define INCLUDE_TLBM_DEFINTIONS_H_
using real = double;
#define MPI_DTYPE MPI_DOUBLE
#endif
