// dropout.cu -- dropout concealment and dropout-mask raster, sm_103a.
//
// Concealment applies a frame's planned line operations (dropout_plan.cpp)
// to its two fields in device memory, in the reference's order
// (DropoutCorrector::correctField / correctDropOut,
// src/dropout/dropout_corrector.cpp:117-157, 469-530): a later operation may
// read a line an earlier one rewrote, so one block owns a frame and runs its
// operations one after another, the block's threads splitting each line.
// The low/high-frequency blend uses the reference's 5-tap luma FIR -- the PAL
// taps, or the NTSC taps the reference also uses for PAL-M
// (src/dropout/luma_filters.cpp:27-38, dropout_corrector.cpp:498-506) --
// evaluated the way FIRFilter::apply
// does (src/decoders/filter/firfilter.h:52-99): FP64 accumulation in tap
// order with zero outside the line, each product and sum rounded separately,
// then truncation to uint16; the final update is modular uint16 arithmetic.
#include <cstdint>
#include <cuda_runtime.h>

#include "dropout_plan.h"

namespace chdg {

__constant__ double c_luma_fir[2][5] = {{0.03283437, 0.23959832, 0.45513461, 0.23959832, 0.03283437},
                                         {0.03275786, 0.23955702, 0.45537024, 0.23955702, 0.03275786}};

__device__ __forceinline__ uint16_t luma_fir(const uint16_t *line, int fw, int x, int taps)
{
    double v = 0.0;
#pragma unroll
    for (int j = 0; j < 5; j++) {
        const int k = x - 2 + j;
        if (k >= 0 && k < fw) v = __dadd_rn(v, __dmul_rn(c_luma_fir[taps][j], (double)line[k]));
    }
    return (uint16_t)__double2uint_rz(v);
}

// frames: per planned frame, the device field index of its slot 0 (slot 1
// is the next field); ops[op_begin[b] .. op_begin[b+1]) are frame b's.
// extras: the batch's extra-capture fields (same stride), which ops with
// srcExtra / chrExtra >= 0 read their replacement lines from.
__global__ void dropout_apply_kernel(uint16_t *fields, long long field_stride, int fw, const int *frames,
                                     const DropOp *ops, const int *op_begin, const uint16_t *extras, int taps)
{
    const int b = blockIdx.x;
    uint16_t *base = fields + (long long)frames[b] * field_stride;
    for (int i = op_begin[b]; i < op_begin[b + 1]; i++) {
        const DropOp op = ops[i];
        uint16_t *target = base + (long long)op.field * field_stride + (long long)op.line * fw;
        const uint16_t *src = (op.srcExtra >= 0 ? extras + (long long)op.srcExtra * field_stride
                                                : base + (long long)op.srcField * field_stride) +
                              (long long)op.srcLine * fw;
        const int x0 = max(op.startx, 0), x1 = min(op.endx, fw);
        if (op.mode == 1) {
            for (int x = x0 + (int)threadIdx.x; x < x1; x += blockDim.x) target[x] = src[x];
        } else {
            const uint16_t *chr = (op.chrExtra >= 0 ? extras + (long long)op.chrExtra * field_stride
                                                    : base + (long long)op.chrField * field_stride) +
                                  (long long)op.chrLine * fw;
            for (int x = x0 + (int)threadIdx.x; x < x1; x += blockDim.x) {
                const uint16_t lf = luma_fir(src, fw, x, taps);
                const uint16_t lfc = luma_fir(chr, fw, x, taps);
                target[x] = (uint16_t)((int)lf + ((int)chr[x] - (int)lfc));
            }
        }
        __syncthreads();
    }
}

// ntsc_taps: the NTSC / PAL-M luma filter instead of PAL's
int dropout_apply(uint16_t *fields, long long field_stride, int fw, const int *d_frames, const DropOp *d_ops,
                  const int *d_op_begin, int nframes, const uint16_t *extras, bool ntsc_taps, cudaStream_t s)
{
    if (nframes <= 0) return 0;
    dropout_apply_kernel<<<nframes, 256, 0, s>>>(fields, field_stride, fw, d_frames, d_ops, d_op_begin, extras,
                                                 ntsc_taps ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// One block per span: x in [x_start, x_end) of row y set to the mask value.
__global__ void mask_raster_kernel(void *plane, int is_float, int width, const Span *spans)
{
    const Span s = spans[blockIdx.x];
    for (int x = s.x_start + (int)threadIdx.x; x < s.x_end; x += blockDim.x) {
        const long long e = (long long)s.y * width + x;
        if (is_float) static_cast<float *>(plane)[e] = 1.0f;
        else static_cast<uint16_t *>(plane)[e] = 0xFFFF;
    }
}

int mask_raster(void *d_plane, bool is_float, int width, int height, const Span *d_spans, int nspans, cudaStream_t s)
{
    const size_t bytes = (size_t)width * height * (is_float ? sizeof(float) : sizeof(uint16_t));
    if (cudaMemsetAsync(d_plane, 0, bytes, s) != cudaSuccess) return -1;
    if (nspans > 0) mask_raster_kernel<<<nspans, 128, 0, s>>>(d_plane, is_float ? 1 : 0, width, d_spans);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace chdg
