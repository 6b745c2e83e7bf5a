// Typed volumes: samples of the VTK scalar types the reference reads
// (char, short, unsigned_short, int, float, double; flyingEdges/util/
// ConvertBuffer.h:45-72, LoadImage.h:168-198), plus unsigned char, converted
// to float32 on the device.  The reference converts every sample with a C
// cast to scalar_t (float) before extracting; (float)v here is the same
// round-to-nearest conversion, so the extraction that follows sees the same
// floats.  Moving the narrow samples and converting on the device divides
// the host -> device bytes of a volume by 4 (8-bit) or 2 (16-bit).
#include <cstdint>

#include "../../include/miniiso.h"
#include "iso_device.cuh"
#include "iso_kernels.h"

namespace iso {

template <typename T>
__global__ void __launch_bounds__(kThreads) k_to_float(const T* __restrict__ in, float* __restrict__ out, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) out[q] = (float)in[q];
}

size_t dtype_bytes(int dtype)
{
    switch (dtype) {
        case ISO_FLOAT32: return 4;
        case ISO_INT8: return 1;
        case ISO_UINT8: return 1;
        case ISO_INT16: return 2;
        case ISO_UINT16: return 2;
        case ISO_INT32: return 4;
        case ISO_FLOAT64: return 8;
    }
    return 0;
}

void launch_to_float(const void* in, int dtype, float* out, long long n, int nsm, cudaStream_t s)
{
    if (n <= 0) return;
    long long blocks = (n + kThreads - 1) / kThreads;
    if (blocks > 16ll * nsm) blocks = 16ll * nsm;
    const unsigned nb = (unsigned)blocks;
    switch (dtype) {
        case ISO_INT8: k_to_float<int8_t><<<nb, kThreads, 0, s>>>(static_cast<const int8_t*>(in), out, n); break;
        case ISO_UINT8: k_to_float<uint8_t><<<nb, kThreads, 0, s>>>(static_cast<const uint8_t*>(in), out, n); break;
        case ISO_INT16: k_to_float<int16_t><<<nb, kThreads, 0, s>>>(static_cast<const int16_t*>(in), out, n); break;
        case ISO_UINT16:
            k_to_float<uint16_t><<<nb, kThreads, 0, s>>>(static_cast<const uint16_t*>(in), out, n);
            break;
        case ISO_INT32: k_to_float<int32_t><<<nb, kThreads, 0, s>>>(static_cast<const int32_t*>(in), out, n); break;
        case ISO_FLOAT64: k_to_float<double><<<nb, kThreads, 0, s>>>(static_cast<const double*>(in), out, n); break;
        default: k_to_float<float><<<nb, kThreads, 0, s>>>(static_cast<const float*>(in), out, n); break;
    }
}

}  // namespace iso
