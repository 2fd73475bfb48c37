// Stage kernels for N = 7 solution points per direction.
#define CHORUS_N 7
#include "kernels_inst.cuh"
