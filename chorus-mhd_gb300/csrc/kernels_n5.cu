// Stage kernels for N = 5 solution points per direction.
#define CHORUS_N 5
#include "kernels_inst.cuh"
