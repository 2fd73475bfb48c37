// Stage kernels for N = 8 solution points per direction.
#define CHORUS_N 8
#include "kernels_inst.cuh"
