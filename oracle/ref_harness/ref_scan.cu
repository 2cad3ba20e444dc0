// ORACLE support (test infrastructure): the prefix sum runSzs runs between
// bitshuffleAndBitflag and encodeDebug -- cub::DeviceScan::ExclusiveSum over the u32
// chunk flags (fz.cu:187-192) -- called the same way, from the CUB that ships with the
// CUDA toolkit (the reference takes the system CUB, lorenzo_var.cuh:17-23).  Used by
// tests/golden/refpipe.py to time and check the reference's own GPU pipeline.
#include <cub/device/device_scan.cuh>

#include <cstdint>

extern "C" {

// Temporary storage CUB wants for m items (the first ExclusiveSum call of fz.cu:189).
int ref_scan_temp_bytes(int m, size_t* bytes)
{
    return (int)cub::DeviceScan::ExclusiveSum(nullptr, *bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr, m);
}

// The scan itself (fz.cu:191), on `stream`.
int ref_scan(void* temp, size_t bytes, const uint32_t* in, uint32_t* out, int m, cudaStream_t stream)
{
    return (int)cub::DeviceScan::ExclusiveSum(temp, bytes, in, out, m, stream);
}

}  // extern "C"
