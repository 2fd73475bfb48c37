// Stage kernels for N = 3 solution points per direction.
#define CHORUS_N 3
#include "kernels_inst.cuh"
