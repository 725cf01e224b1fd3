// greens_quadrature.cu -- the element-wise front of the Green's-function consumers
// (multimode.py:15-47): from the bosonic transfer matrices C and S (a_out = C a + S a^dagger), the
// quadrature-basis matrix Z and the a-basis block matrix whose products give the covariance matrices.
// Both kernels are HBM-bound copies with arithmetic (32 B read, 32 B written per element of C); the
// grid strides over the elements of C so that consecutive threads read and write consecutive columns.
#include <algorithm>
#include <cstdint>

#include "nlm_device.cuh"
#include "nlm_kernels.h"

namespace nlm {

// Z (2 rows x 2 cols, row-major) = [[Re(C + S), -Im(C - S)], [Im(C + S), Re(C - S)]].  Each thread
// takes two adjacent columns, so that the four stores are 16-byte pairs (cols even; the pairs start
// at even element offsets, 16-byte aligned for a 16-byte aligned Z).
__global__ void k_quadrature_z2(const double2* __restrict__ C, const double2* __restrict__ S, long long rows,
                                long long cols, double* __restrict__ Z) {
  const long long half = cols / 2, total = rows * half, zc = 2 * cols;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long r = idx / half, c = 2 * (idx - r * half);
    const long long e = r * cols + c;
    const double2 c0 = __ldg(C + e), c1 = __ldg(C + e + 1), s0 = __ldg(S + e), s1 = __ldg(S + e + 1);
    double2* top = reinterpret_cast<double2*>(Z + r * zc + c);
    double2* bottom = reinterpret_cast<double2*>(Z + (rows + r) * zc + c);
    top[0] = make_double2(c0.x + s0.x, c1.x + s1.x);
    top[half] = make_double2(-(c0.y - s0.y), -(c1.y - s1.y));
    bottom[0] = make_double2(c0.y + s0.y, c1.y + s1.y);
    bottom[half] = make_double2(c0.x - s0.x, c1.x - s1.x);
  }
}

// The same one column per thread, for odd column counts.
__global__ void k_quadrature_z(const double2* __restrict__ C, const double2* __restrict__ S, long long rows,
                               long long cols, double* __restrict__ Z) {
  const long long total = rows * cols, zc = 2 * cols;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long r = idx / cols, c = idx - r * cols;
    const double2 cv = __ldg(C + idx), sv = __ldg(S + idx);
    double* top = Z + r * zc + c;
    double* bottom = Z + (rows + r) * zc + c;
    top[0] = cv.x + sv.x;
    top[cols] = -(cv.y - sv.y);
    bottom[0] = cv.y + sv.y;
    bottom[cols] = cv.x - sv.x;
  }
}

// Za (2 rows x 2 cols complex, row-major) = sqrt(1/2) [[C, S], [conj(S), conj(C)]]
__global__ void k_abasis_z(const double2* __restrict__ C, const double2* __restrict__ S, long long rows, long long cols,
                           double2* __restrict__ Za) {
  const double h = 0.7071067811865476;   // sqrt(1/2) rounded to double, as numpy's np.sqrt(1 / 2)
  const long long total = rows * cols, zc = 2 * cols;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long r = idx / cols, c = idx - r * cols;
    const double2 cv = __ldg(C + idx), sv = __ldg(S + idx);
    double2* top = Za + r * zc + c;
    double2* bottom = Za + (rows + r) * zc + c;
    top[0] = make_double2(cv.x * h, cv.y * h);
    top[cols] = make_double2(sv.x * h, sv.y * h);
    bottom[0] = make_double2(sv.x * h, -sv.y * h);
    bottom[cols] = make_double2(cv.x * h, -cv.y * h);
  }
}

static int stride_grid(long long total) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (total + 255) / 256;
  return (int)std::max<long long>(1, std::min<long long>(want, 8LL * sms));
}

cudaError_t launch_quadrature_z(const double2* C, const double2* S, long long rows, long long cols, double* Z,
                                cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  if (cols % 2 == 0 && reinterpret_cast<uintptr_t>(Z) % 16 == 0)
    k_quadrature_z2<<<stride_grid(rows * cols / 2), 256, 0, s>>>(C, S, rows, cols, Z);
  else
    k_quadrature_z<<<stride_grid(rows * cols), 256, 0, s>>>(C, S, rows, cols, Z);
  return cudaGetLastError();
}

cudaError_t launch_abasis_z(const double2* C, const double2* S, long long rows, long long cols, double2* Za,
                            cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  k_abasis_z<<<stride_grid(rows * cols), 256, 0, s>>>(C, S, rows, cols, Za);
  return cudaGetLastError();
}

}  // namespace nlm
