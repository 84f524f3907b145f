// 16-bit field codes of the alpha driver's output files (Dtype2B_E and
// Dtype2B_CI, source_beta_to_alpha/src/anisotropic_hip.c:3920-3944): every
// cell of the block, order parameters as (eta + 0.1) * 30000 and
// concentrations as c * 50000, computed in FP64 and truncated toward zero.
// The reference's conversion is undefined outside [0, 65535]; here the code
// saturates at the ends of that range (NaN gives 0).
#include "sclet_internal.cuh"

namespace sclet {

namespace {

template <typename T>
__global__ void u16_kernel(const T *__restrict__ u, double shift, double offset, double scale, long long cells,
                           unsigned short *__restrict__ out) {
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < cells; l += (long long)gridDim.x * blockDim.x) {
    const double v = ((double)u[l] + shift + offset) * scale;
    double t = trunc(v);
    t = t > 65535.0 ? 65535.0 : t;
    t = t >= 0.0 ? t : 0.0;  // also maps NaN to 0
    out[l] = (unsigned short)t;
  }
}

}  // namespace

template <typename T>
cudaError_t launch_field_u16(const T *u, int kind, double shift, long long cells, unsigned short *out, cudaStream_t s) {
  const double offset = kind == 0 ? 0.1 : 0.0, scale = kind == 0 ? 30000.0 : 50000.0;
  long long b = (cells + 255) / 256;
  u16_kernel<T><<<(int)(b > 152 * 16 ? 152 * 16 : b), 256, 0, s>>>(u, shift, offset, scale, cells, out);
  launch_counter()++;
  return cudaGetLastError();
}

template cudaError_t launch_field_u16<double>(const double *, int, double, long long, unsigned short *, cudaStream_t);
template cudaError_t launch_field_u16<float>(const float *, int, double, long long, unsigned short *, cudaStream_t);

}  // namespace sclet
