// Stage kernels for N = 2 solution points per direction.
#define CHORUS_N 2
#include "kernels_inst.cuh"
