// Stage kernels for N = 4 solution points per direction.
#define CHORUS_N 4
#include "kernels_inst.cuh"
