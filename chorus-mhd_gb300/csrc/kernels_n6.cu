// Stage kernels for N = 6 solution points per direction.
#define CHORUS_N 6
#include "kernels_inst.cuh"
