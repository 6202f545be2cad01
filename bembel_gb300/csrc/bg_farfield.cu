// Far-field assembly on GB300: the interpolation points of every cluster
// (interpolationPoints2D / map2surface, H2Multipole.hpp:324-375) and the FP64
// coupling blocks F_ij = k(x_i, y_j) |J(x_i)| |J(y_j)| of the low-rank leaves
// (Laplace/Helmholtz SingleLayerOperator::evaluateFMMInterpolation_impl, :87-110).
#include "bg_kernels.cuh"

namespace bg {

constexpr double kInv4PiF = 0.07957747154594767;

// out32 holds the point relative to the cluster centre (centres[c], FP64), so
// that FP32 differences of nearby-but-admissible clusters keep full relative
// accuracy once the FP64 centre difference is added back.
template <int G>
__global__ void k_cluster_points(PatchTable pt, int level, int nclusters, const double* __restrict__ cheb, int np,
                                 const d4* __restrict__ centres, d4* __restrict__ out64, float4* __restrict__ out32,
                                 double* __restrict__ tan64, float* __restrict__ tan32) {
  const int np2 = np * np;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nclusters * np2) return;
  const int c = (int)(idx / np2), q = (int)(idx % np2);
  const int per_patch = 1 << (2 * level);
  const int patch = c / per_patch;
  int local = c % per_patch, ix = 0, iy = 0;
  for (int b = level - 1; b >= 0; --b) {
    const int d = (local >> (2 * b)) & 3;
    ix = 2 * ix + (d == 1 || d == 2);
    iy = 2 * iy + (d == 2 || d == 3);
  }
  const double H = 1.0 / double(1 << level);
  double x[3], dx[3], dy[3];
  surface_frame<G>(pt, patch, ix * H + H * cheb[q / np], iy * H + H * cheb[q % np], x, dx, dy);
  // Maxwell couples with the bare kernel and carries the tangents instead
  const double kap = tan64 ? 1.0 : surface_measure(dx, dy);
  out64[idx] = d4{x[0], x[1], x[2], kap};
  if (tan64) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      tan64[6 * idx + k] = dx[k];
      tan64[6 * idx + 3 + k] = dy[k];
      tan32[6 * idx + k] = (float)dx[k];
      tan32[6 * idx + 3 + k] = (float)dy[k];
    }
  }
  if (out32) {
    const d4 cen = centres[c];
    out32[idx] = make_float4((float)(x[0] - cen.x), (float)(x[1] - cen.y), (float)(x[2] - cen.z), (float)kap);
  }
}

cudaError_t launch_cluster_points(int G, const PatchTable& pt, int level, int nclusters, const double* cheb, int np,
                                  const d4* centres, d4* out64, float4* out32, double* tan64, float* tan32,
                                  cudaStream_t s) {
  const long n = (long)nclusters * np * np;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if ((tan64 == nullptr) != (tan32 == nullptr)) return cudaErrorInvalidValue;
  switch (G) {
    case 2: k_cluster_points<2><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32, tan64, tan32); break;
    case 3: k_cluster_points<3><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32, tan64, tan32); break;
    case 4: k_cluster_points<4><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32, tan64, tan32); break;
    case 5: k_cluster_points<5><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32, tan64, tan32); break;
    case 6: k_cluster_points<6><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32, tan64, tan32); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// One CTA per block: stage both clusters' points, write F column-major.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_far_assemble(const d4* __restrict__ pts, const int2* __restrict__ pairs,
                                                      int B, long bstride, double kre, double kim,
                                                      double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  d4* xs = reinterpret_cast<d4*>(smem_raw);
  d4* ys = xs + B;
  const int2 pr = pairs[blockIdx.x];
  for (int q = threadIdx.x; q < B; q += blockDim.x) {
    xs[q] = pts[(long)pr.x * B + q];
    ys[q] = pts[(long)pr.y * B + q];
  }
  __syncthreads();
  const long base = (long)blockIdx.x * bstride;
  for (int e = threadIdx.x; e < B * B; e += blockDim.x) {
    const int i = e % B, j = e / B;
    const d4 x = xs[i], y = ys[j];
    const double d0 = x.x - y.x, d1 = x.y - y.y, d2 = x.z - y.z;
    const double r2 = fma(d0, d0, fma(d1, d1, d2 * d2));
    const double inv = rsqrt_nr(r2);
    const double amp = inv * kInv4PiF * x.w * y.w;
    if (!CPLX) {
      out[base + e] = amp;
    } else {
      const double r = r2 * inv;
      double sn, cs;
      sincos(kre * r, &sn, &cs);
      double a = amp;
      if (kim != 0.0) a *= exp(kim * r);
      reinterpret_cast<double2*>(out)[base + e] = make_double2(cs * a, -sn * a);
    }
  }
}

cudaError_t launch_far_assemble(bool cplx, const d4* pts, const int2* pairs, int nblocks, int B, long bstride,
                                double kre, double kim, void* out, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  const size_t smem = 2 * B * sizeof(d4);
  if (cplx) k_far_assemble<true><<<nblocks, 256, smem, s>>>(pts, pairs, B, bstride, kre, kim, static_cast<double*>(out));
  else k_far_assemble<false><<<nblocks, 256, smem, s>>>(pts, pairs, B, bstride, kre, kim, static_cast<double*>(out));
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Maxwell far field around the scalar kernel product. One thread per
// (cluster, point, right-hand side of the chunk); the three channels of Y and
// Z are [channel][cluster][np2][nrhs].
template <typename S, typename R>
__global__ void k_mw_far_in(int ncl, int np2, const S* __restrict__ y, int nrhs, int r0, int nr,
                            const R* __restrict__ tan, S* __restrict__ yv) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ncl * np2 * nr) return;
  const int r = (int)(idx % nr);
  const long cj = idx / nr;  // cluster * np2 + j
  const long ch = (long)ncl * np2 * nrhs;  // one channel
  const long row = cj * nrhs + r0 + r;
  const S p0 = y[row], p1 = y[ch + row], dv = y[2 * ch + row];
  const R* t = tan + 6 * cj;
  S* o = yv + cj * 4 * nr + r;
#pragma unroll
  for (int q = 0; q < 3; ++q) o[q * nr] = p0 * t[q] + p1 * t[3 + q];
  o[3 * nr] = dv;
}

template <typename S, typename R>
__global__ void k_mw_far_out(int ncl, int np2, const S* __restrict__ zv, int nrhs, int r0, int nr,
                             const R* __restrict__ tan, S m, S* __restrict__ z) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)ncl * np2 * nr) return;
  const int r = (int)(idx % nr);
  const long ci = idx / nr;
  const long ch = (long)ncl * np2 * nrhs;
  const long row = ci * nrhs + r0 + r;
  const R* t = tan + 6 * ci;
  const S* v = zv + ci * 4 * nr + r;
  const S v0 = v[0], v1 = v[nr], v2 = v[2 * nr];
  z[row] = v0 * t[0] + v1 * t[1] + v2 * t[2];
  z[ch + row] = v0 * t[3] + v1 * t[4] + v2 * t[5];
  z[2 * ch + row] = v[3 * nr] * m;
}

cudaError_t launch_mw_far_in(int S, int ncl, int np2, const void* y, int nrhs, int r0, int nr, const void* tan,
                             void* yv, cudaStream_t s) {
  const long n = (long)ncl * np2 * nr;
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (S == 1)
    k_mw_far_in<cd, double><<<grid, 256, 0, s>>>(ncl, np2, (const cd*)y, nrhs, r0, nr, (const double*)tan, (cd*)yv);
  else if (S == 3)
    k_mw_far_in<cf, float><<<grid, 256, 0, s>>>(ncl, np2, (const cf*)y, nrhs, r0, nr, (const float*)tan, (cf*)yv);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_mw_far_out(int S, int ncl, int np2, const void* zv, int nrhs, int r0, int nr, const void* tan,
                              double mre, double mim, void* z, cudaStream_t s) {
  const long n = (long)ncl * np2 * nr;
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (S == 1)
    k_mw_far_out<cd, double><<<grid, 256, 0, s>>>(ncl, np2, (const cd*)zv, nrhs, r0, nr, (const double*)tan,
                                                  cd{mre, mim}, (cd*)z);
  else if (S == 3)
    k_mw_far_out<cf, float><<<grid, 256, 0, s>>>(ncl, np2, (const cf*)zv, nrhs, r0, nr, (const float*)tan,
                                                 cf{(float)mre, (float)mim}, (cf*)z);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace bg
