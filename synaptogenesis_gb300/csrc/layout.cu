// Device-side conversions between the host layout of per-synapse arrays
// ([rows][cols], the reference's CPU layout) and the device layouts (banded
// or transposed, csrc/state.h), run on the state's stream around the
// uploads and downloads so that the host only copies contiguous memory.
#include <cuda_runtime.h>

#include <cstdint>

#include "cuda_check.h"
#include "state.h"

namespace sg {
namespace {

// host [rows][cols] -> banded [rows/8][cols][8] (padding rows zero); one
// thread per banded element, so consecutive threads write consecutive words.
__global__ void k_to_bands(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int rows,
                           int cols, long long n_out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_out) return;
    const long long band = o / ((long long)cols * kBand);
    const long long rem = o - band * cols * kBand;
    const int c = (int)(rem / kBand), rr = (int)(rem % kBand);
    const long long r = band * kBand + rr;
    out[o] = r < rows ? in[r * cols + c] : 0u;
}

__global__ void k_from_bands(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int rows,
                             int cols, long long n_in) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_in) return;
    const long long band = o / ((long long)cols * kBand);
    const long long rem = o - band * cols * kBand;
    const int c = (int)(rem / kBand), rr = (int)(rem % kBand);
    const long long r = band * kBand + rr;
    if (r < rows) out[r * cols + c] = in[o];
}

// [rows][cols] -> [cols][rows] through 32 x 32 shared-memory tiles.
__global__ void k_transpose(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int rows,
                            int cols) {
    __shared__ uint32_t t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[(size_t)c * rows + r] = t[threadIdx.x][i];
    }
}

unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

void launch_to_bands(const uint32_t* in, uint32_t* out, int rows, int cols, size_t dev_count,
                     cudaStream_t s) {
    if (dev_count == 0) return;
    k_to_bands<<<blocks((long long)dev_count), 256, 0, s>>>(in, out, rows, cols, (long long)dev_count);
    SG_LAUNCH_CHECK();
}

void launch_from_bands(const uint32_t* in, uint32_t* out, int rows, int cols, size_t dev_count,
                       cudaStream_t s) {
    if (dev_count == 0) return;
    k_from_bands<<<blocks((long long)dev_count), 256, 0, s>>>(in, out, rows, cols,
                                                             (long long)dev_count);
    SG_LAUNCH_CHECK();
}

void launch_transpose(const uint32_t* in, uint32_t* out, int rows, int cols, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return;
    const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
    k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, out, rows, cols);
    SG_LAUNCH_CHECK();
}

}  // namespace sg
