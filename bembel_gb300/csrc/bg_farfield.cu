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
                                 const d4* __restrict__ centres, d4* __restrict__ out64, float4* __restrict__ out32) {
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
  const double kap = surface_measure(dx, dy);
  out64[idx] = d4{x[0], x[1], x[2], kap};
  if (out32) {
    const d4 cen = centres[c];
    out32[idx] = make_float4((float)(x[0] - cen.x), (float)(x[1] - cen.y), (float)(x[2] - cen.z), (float)kap);
  }
}

cudaError_t launch_cluster_points(int G, const PatchTable& pt, int level, int nclusters, const double* cheb, int np,
                                  const d4* centres, d4* out64, float4* out32, cudaStream_t s) {
  const long n = (long)nclusters * np * np;
  const unsigned grid = (unsigned)((n + 127) / 128);
  switch (G) {
    case 2: k_cluster_points<2><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32); break;
    case 3: k_cluster_points<3><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32); break;
    case 4: k_cluster_points<4><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32); break;
    case 5: k_cluster_points<5><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32); break;
    case 6: k_cluster_points<6><<<grid, 128, 0, s>>>(pt, level, nclusters, cheb, np, centres, out64, out32); break;
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

}  // namespace bg
