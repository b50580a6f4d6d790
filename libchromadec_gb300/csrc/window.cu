// window.cu -- black padding fields of a decode window, and the black tail of
// a shifted subcarrier-locked second field, on the device.
//
// Frames outside the capture (and frames whose metadata is unusable) enter
// the Transform-PAL window as fields filled with the black level
// (SourceField::loadFields, src/decoders/source_field.cpp:147-158). Window
// fields start 128-byte aligned, so each thread writes 8 samples at a time.
#include <cstdint>
#include <cuda_runtime.h>

namespace chdg {

__global__ void fill_fields_kernel(uint16_t *fields, long long field_stride, long long field_len, uint16_t value)
{
    uint16_t *f = fields + (long long)blockIdx.y * field_stride;
    const unsigned v2 = (unsigned)value | ((unsigned)value << 16);
    const uint4 v8 = make_uint4(v2, v2, v2, v2);
    const long long n8 = field_len / 8;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n8; i += (long long)gridDim.x * blockDim.x)
        reinterpret_cast<uint4 *>(f)[i] = v8;
    const long long tail = field_len - 8 * n8;
    if (blockIdx.x == 0 && threadIdx.x < tail) f[8 * n8 + threadIdx.x] = value;
}

int fill_fields(uint16_t *fields, long long field_stride, long long field_len, int nfields, uint16_t value,
                cudaStream_t s)
{
    if (nfields <= 0) return 0;
    if ((reinterpret_cast<uintptr_t>(fields) & 15) != 0 || (field_stride & 7) != 0) return -1;
    fill_fields_kernel<<<dim3(64, (unsigned)nfields), 256, 0, s>>>(fields, field_stride, field_len, value);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void fill_samples_kernel(uint16_t *p, long long n, uint16_t value)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = value;
}

// Any run of samples, no alignment needed (the 2 black samples a shifted
// second field ends with).
int fill_samples(uint16_t *p, long long n, uint16_t value, cudaStream_t s)
{
    if (n <= 0) return 0;
    const unsigned blocks = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    fill_samples_kernel<<<blocks, 256, 0, s>>>(p, n, value);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace chdg
