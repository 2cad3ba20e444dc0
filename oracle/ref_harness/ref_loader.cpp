// ORACLE support (test infrastructure): launches the reference's own kernels from
// oracle/_ref/ref_kernels.fatbin with the reference's launch shapes, so that fixtures
// of their outputs can pin the oracle.  Used only by tests/golden/make_golden.py.
//
//   c_lorenzo_{1d,2d,3d}   grids/blocks of launch_construct_LorenzoI_var
//                          (lorenzo_var.cuh:530-585)
//   bitshuffleAndBitflag   grid floor(len/2048), block (32,32)       (fz.cu:172-174)
//   encodeDebug            grid ceil(2 len/512), block 32            (fz.cu:205)
#include <cuda.h>

#include <cstdint>
#include <cstring>

namespace {
CUmodule   g_mod = nullptr;
CUfunction g_fn[5] = {};  // lorenzo 1d, 2d, 3d, bitshuffle, encode
const char* kNames[5] = {"c_lorenzo_1d1l", "c_lorenzo_2d1l", "c_lorenzo_3d1l",
                         "bitshuffleAndBitflag", "encodeDebug"};

struct Dim3 {
    unsigned x, y, z;
};
}  // namespace

extern "C" {

// Loads the fatbin into the current (primary) context of device 0 and finds the
// kernels by name.  Returns 0 on success, a CUresult or -1 (kernel missing) otherwise.
int ref_load(const char* path)
{
    CUresult r = cuInit(0);
    if (r != CUDA_SUCCESS) return r;
    CUdevice dev;
    CUcontext ctx;
    if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return r;
    if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return r;
    if ((r = cuCtxSetCurrent(ctx)) != CUDA_SUCCESS) return r;
    if ((r = cuModuleLoad(&g_mod, path)) != CUDA_SUCCESS) return r;
    unsigned count = 0;
    if ((r = cuModuleGetFunctionCount(&count, g_mod)) != CUDA_SUCCESS) return r;
    CUfunction fns[256];
    if (count > 256) count = 256;
    if ((r = cuModuleEnumerateFunctions(fns, count, g_mod)) != CUDA_SUCCESS) return r;
    for (unsigned i = 0; i < count; ++i) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, fns[i]) != CUDA_SUCCESS || !name) continue;
        for (int k = 0; k < 5; ++k)
            if (std::strstr(name, kNames[k])) g_fn[k] = fns[i];
    }
    for (int k = 0; k < 5; ++k)
        if (!g_fn[k]) return -1;
    return 0;
}

int ref_c_lorenzo(int nd, float* data, uint16_t* quant, uint8_t* signum, unsigned x, unsigned y,
                  unsigned z, float ebx2_r, CUstream s)
{
    Dim3  len3{x, y, z}, leap3{1, x, x * y};
    void* args[] = {&data, &quant, &signum, &len3, &leap3, &ebx2_r};
    auto  pd     = [](unsigned l, unsigned b) { return (l - 1) / b + 1; };
    if (nd == 1) return cuLaunchKernel(g_fn[0], pd(x, 256), pd(y, 1), pd(z, 1), 64, 1, 1, 0, s, args, nullptr);
    if (nd == 2) return cuLaunchKernel(g_fn[1], pd(x, 16), pd(y, 16), pd(z, 1), 16, 2, 1, 0, s, args, nullptr);
    return cuLaunchKernel(g_fn[2], pd(x, 32), pd(y, 8), pd(z, 8), 32, 1, 8, 0, s, args, nullptr);
}

int ref_bitshuffle(uint32_t* in, uint32_t* out, unsigned len, uint32_t* bitflag, uint32_t* byteflag,
                   CUstream s)
{
    unsigned grid = len / 2048;
    if (grid == 0) return 0;  // the reference's launch with a zero grid does nothing
    int   block_size = 16;
    void* args[]     = {&in, &out, &block_size, &bitflag, &byteflag};
    return cuLaunchKernel(g_fn[3], grid, 1, 1, 32, 32, 1, 0, s, args, nullptr);
}

int ref_encode(uint8_t* in, uint8_t* out, uint32_t* presum, unsigned len, CUstream s)
{
    unsigned nl  = len * 2;
    unsigned dcs = nl % 512 == 0 ? nl / 512 : nl / 512 + 1;
    int      block_size = 16;
    void*    args[]     = {&block_size, &in, &out, &presum};
    return cuLaunchKernel(g_fn[4], dcs, 1, 1, 32, 1, 1, 0, s, args, nullptr);
}

}  // extern "C"
