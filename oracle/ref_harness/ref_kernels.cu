// ORACLE support (test infrastructure): the reference's own kernels, compiled from the
// FZ-GPU sources into oracle/_ref/ref_kernels.fatbin (oracle/Makefile, target `ref`).
// Nothing of the reference is copied here: this translation unit only includes its
// fz.cu (with main renamed) and instantiates the three Lorenzo kernel templates that
// launch_construct_LorenzoI_var dispatches to (lorenzo_var.cuh:571-585).  The kernels
// are loaded by name and launched by oracle/ref_harness/ref_loader.cpp.
#define main fz_reference_main
#include "fz.cu"
#undef main

template __global__ void cusz::experimental::c_lorenzo_1d1l<float, uint16_t, float, 256, 4>(
    float*, uint16_t*, bool*, dim3, dim3, float);
template __global__ void cusz::experimental::c_lorenzo_2d1l_16x16data_mapto16x2<float, uint16_t, float>(
    float*, uint16_t*, bool*, dim3, dim3, float);
template __global__ void cusz::experimental::c_lorenzo_3d1l_32x8x8data_mapto32x1x8<float, uint16_t, float>(
    float*, uint16_t*, bool*, dim3, dim3, float);
