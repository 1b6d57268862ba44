// Exhaustive (separate laser and detector points) volume renderer and its
// adjoint with respect to the volume.
//
// Reference: src/render/volume_cuda.cu:298-377 (forward, one thread per
// (voxel column, scan point, laser point) with global atomics) and :415-466
// (gradient: an empty kernel). Here the forward gives each CTA one scan point
// and a tile of laser points, walks the occupied voxels and splats each
// voxel's path-length interval into a shared [T][tile] histogram that is
// flushed with row stores; the adjoint (the forward is linear in the volume)
// gathers per voxel.
#include <string>

#include "capi_common.cuh"
#include "tune.cuh"

namespace totri {
namespace vexh {

struct Geo {
  int D, H, W, S, L, T;
  float sx, sy, sz, ex, ey, ez, bw, bo;
};

struct Pts {  // [B, 3, n] with strides
  const float* p;
  int64_t sb, sc, sn;
  __device__ fv3 at(int b, int i) const {
    const float* q = p + b * sb + i * sn;
    return mkv(q[0], q[sc], q[2 * sc]);
  }
};

struct Interval {
  bool ok;
  int first, last;
  float bf0, bf1, range;
};

// Path-length interval of voxel (xi, yi, zi) for the pair (s, l), binned
// (volume_cuda.cu:314-364); FP32 decisions as in the oracle.
__device__ __forceinline__ Interval interval(const Geo& g, fv3 sc, fv3 lc, int xi, int yi,
                                             int zi) {
  Interval r{false, 0, 0, 0.f, 0.f, 0.f};
  const float xf = xadd(g.sx, xmul(xdiv(xadd((float)xi, 0.5f), (float)g.W), xsub(g.ex, g.sx)));
  const float yf = xadd(g.sy, xmul(xdiv(xadd((float)yi, 0.5f), (float)g.H), xsub(g.ey, g.sy)));
  const float zf = xadd(g.sz, xmul(xdiv(xadd((float)zi, 0.5f), (float)g.D), xsub(g.ez, g.sz)));
  const float half = xmul(xdiv(0.5f, (float)g.D), xsub(g.ez, g.sz));
  const float zf0 = xsub(zf, half), zf1 = xadd(zf, half);
  const fv3 p0 = mkv(xf, yf, zf0), p1 = mkv(xf, yf, zf1);
  float d0 = xadd(xlen(xsub3(sc, p0)), xlen(xsub3(lc, p0)));
  float d1 = xadd(xlen(xsub3(sc, p1)), xlen(xsub3(lc, p1)));
  if (d1 < d0) {
    const float t = d0;
    d0 = d1;
    d1 = t;
  }
  float bf0 = xdiv(xsub(d0, g.bo), g.bw), bf1 = xdiv(xsub(d1, g.bo), g.bw);
  const float range = xsub(bf1, bf0);
  int first = (int)floorf(bf0), last = (int)floorf(bf1);
  if (first < 0) {
    if (last < 0) return r;
    bf0 = 0.f;
    first = 0;
  }
  if (last >= g.T) {
    if (first >= g.T) return r;
    bf1 = (float)(g.T - 1);
    last = g.T - 1;
  }
  r.ok = true;
  r.first = first;
  r.last = last;
  r.bf0 = bf0;
  r.bf1 = bf1;
  r.range = range;
  return r;
}

__global__ void compact_kernel(const float* __restrict__ vol, int64_t n, uint32_t* list,
                               uint32_t* count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool occ = i < n && vol[i] != 0.f;
  const uint32_t m = __ballot_sync(0xffffffffu, occ);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (occ) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
}

template <int LT>
__global__ void __launch_bounds__(256) forward_kernel(Geo g, int b, const float* __restrict__ vol,
                                                      const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ count, Pts sp,
                                                      Pts lp, float* __restrict__ out) {
  extern __shared__ float hist[];  // [T][LT]
  const int s = blockIdx.x;
  const int l0 = blockIdx.y * LT;
  for (int j = threadIdx.x; j < g.T * LT; j += blockDim.x) hist[j] = 0.f;
  __syncthreads();
  const uint32_t nnz = *count;
  const int ll = threadIdx.x % LT;
  const int l = l0 + ll;
  if (l < g.L) {
    const fv3 sc = sp.at(b, s), lc = lp.at(b, l);
    for (uint32_t v = threadIdx.x / LT; v < nnz; v += blockDim.x / LT) {
      const uint32_t lin = __ldg(list + v);
      const int xi = (int)(lin % g.W), yi = (int)((lin / g.W) % g.H);
      const int zi = (int)(lin / ((uint32_t)g.W * g.H));
      const Interval iv = interval(g, sc, lc, xi, yi, zi);
      if (!iv.ok) continue;
      const float occ = __ldg(vol + lin);
      float* col = hist + ll;
      if (iv.first == iv.last) {
        atomicAdd(col + iv.first * LT, occ);
        continue;
      }
      const float fo = occ / iv.range;
      atomicAdd(col + iv.first * LT, (1.f - (iv.bf0 - (float)iv.first)) * fo);
      for (int t = iv.first + 1; t < iv.last; ++t) atomicAdd(col + t * LT, fo);
      atomicAdd(col + iv.last * LT, (iv.bf1 - (float)iv.last) * fo);
    }
  }
  __syncthreads();
  // out[b][t][s][l0 .. l0+LT)
  const size_t base = ((size_t)b * g.T * g.S + s) * g.L + l0;
  for (int j = threadIdx.x; j < g.T * LT; j += blockDim.x) {
    const int t = j / LT, c = j - t * LT;
    if (l0 + c < g.L) out[base + (size_t)t * g.S * g.L + c] = hist[j];
  }
}

// d loss / d volume: per voxel, the forward weights against transient_grad.
__global__ void adjoint_kernel(Geo g, int B, Pts sp, Pts lp, const float* __restrict__ tg,
                               float* __restrict__ vg) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (v >= nv * B) return;
  const int b = (int)(v / nv);
  const int64_t lin = v - (int64_t)b * nv;
  const int xi = (int)(lin % g.W), yi = (int)((lin / g.W) % g.H), zi = (int)(lin / ((int64_t)g.W * g.H));
  float acc = 0.f;
  const size_t st = (size_t)g.S * g.L;
  for (int s = 0; s < g.S; ++s) {
    const fv3 sc = sp.at(b, s);
    for (int l = 0; l < g.L; ++l) {
      const Interval iv = interval(g, sc, lp.at(b, l), xi, yi, zi);
      if (!iv.ok) continue;
      const float* col = tg + (size_t)b * g.T * st + (size_t)s * g.L + l;
      if (iv.first == iv.last) {
        acc += __ldg(col + iv.first * st);
        continue;
      }
      float sum = (1.f - (iv.bf0 - (float)iv.first)) * __ldg(col + iv.first * st);
      for (int t = iv.first + 1; t < iv.last; ++t) sum += __ldg(col + t * st);
      sum += (iv.bf1 - (float)iv.last) * __ldg(col + iv.last * st);
      acc += sum / iv.range;
    }
  }
  vg[v] = acc;
}

}  // namespace vexh

namespace {

int check_pts(const totri_array_t* a, const char* name, int64_t B, int64_t& n, vexh::Pts& p) {
  TOTRI_TRY(check_array(a, name, 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(a, name, 0, B));
  TOTRI_TRY(check_dim(a, name, 1, 3));
  n = a->shape[2];
  p = vexh::Pts{static_cast<const float*>(a->data), a->strides[0], a->strides[1], a->strides[2]};
  return TOTRI_OK;
}

template <int LT>
int launch_fwd(const vexh::Geo& g, int b, const float* vol, const uint32_t* list,
               const uint32_t* count, const vexh::Pts& sp, const vexh::Pts& lp, float* out,
               cudaStream_t stream) {
  const size_t smem = sizeof(float) * (size_t)g.T * LT;
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(vexh::forward_kernel<LT>), smem));
  const dim3 grid((unsigned)g.S, (unsigned)ceil_div(g.L, LT));
  TOTRI_KERNEL("volume exhaustive forward", stream,
               vexh::forward_kernel<LT><<<grid, 256, smem, stream>>>(g, b, vol, list, count, sp,
                                                                     lp, out));
  return TOTRI_OK;
}

}  // namespace
}  // namespace totri

using namespace totri;

extern "C" {

int totri_volume_exhaustive_forward(const totri_array_t* vol, const totri_array_t* scan_points,
                                    const totri_array_t* laser_points,
                                    const totri_array_t* scan_origin,
                                    const totri_array_t* laser_origin,
                                    const totri_array_t* transient, const float start[3],
                                    const float end[3], float bw, float bo, void* ws,
                                    size_t ws_bytes, void* stream_) {
  (void)scan_origin;  // unused by the reference kernel (volume_cuda.cu:312-313)
  (void)laser_origin;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(check_array(vol, "volume", 4, -1));
  if (vol->dtype != TOTRI_FLOAT32)
    return fail(TOTRI_ERR_UNSUPPORTED, "volume renderer: only float32 tensors are supported");
  TOTRI_TRY(check_contiguous(vol, "volume"));
  const int64_t B = vol->shape[0];
  int64_t S, L;
  vexh::Pts sp, lp;
  TOTRI_TRY(check_pts(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts(laser_points, "laser_points", B, L, lp));
  TOTRI_TRY(check_array(transient, "transient", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_dim(transient, "transient", 3, L));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  vexh::Geo g{(int)vol->shape[1], (int)vol->shape[2], (int)vol->shape[3], (int)S, (int)L,
              (int)transient->shape[1], start[0], start[1], start[2], end[0], end[1], end[2],
              bw, bo};
  if (numel(transient) == 0) return TOTRI_OK;
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const size_t need = align_up(sizeof(uint32_t) * (nv + 64), 256);
  if (!ws || ws_bytes < need)
    return fail(TOTRI_ERR_WORKSPACE, "workspace of " + std::to_string(need) + " bytes required");
  uint32_t* count = static_cast<uint32_t*>(ws);
  uint32_t* list = count + 64;
  for (int b = 0; b < (int)B; ++b) {
    const float* vb = static_cast<const float*>(vol->data) + (size_t)b * nv;
    TOTRI_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t), stream));
    TOTRI_KERNEL("volume compact", stream,
                 vexh::compact_kernel<<<(unsigned)ceil_div(nv, 256), 256, 0, stream>>>(
                     vb, nv, list, count));
    float* out = static_cast<float*>(transient->data);
    const size_t budget = 200 * 1024;
    const int want = tune::get("volume.exhaustive.lt");
    if (want == 1 || want == 8 || want == 32) {
      if ((size_t)g.T * want * 4 > budget)
        return fail(TOTRI_ERR_INVALID_ARGUMENT, "tuned laser tile too large for the bin count");
      if (want == 32) TOTRI_TRY(launch_fwd<32>(g, b, vb, list, count, sp, lp, out, stream));
      else if (want == 8) TOTRI_TRY(launch_fwd<8>(g, b, vb, list, count, sp, lp, out, stream));
      else TOTRI_TRY(launch_fwd<1>(g, b, vb, list, count, sp, lp, out, stream));
    } else if (want != 0) {
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "laser tile must be 1, 8 or 32");
    } else if ((size_t)g.T * 32 * 4 <= budget && L >= 32)
      TOTRI_TRY(launch_fwd<32>(g, b, vb, list, count, sp, lp, out, stream));
    else if ((size_t)g.T * 8 * 4 <= budget && L >= 8)
      TOTRI_TRY(launch_fwd<8>(g, b, vb, list, count, sp, lp, out, stream));
    else if ((size_t)g.T * 4 <= budget)
      TOTRI_TRY(launch_fwd<1>(g, b, vb, list, count, sp, lp, out, stream));
    else
      return fail(TOTRI_ERR_UNSUPPORTED, "too many bins for one tile");
  }
  return TOTRI_OK;
}

int totri_volume_exhaustive_grad_volume(const totri_array_t* tg,
                                        const totri_array_t* scan_points,
                                        const totri_array_t* laser_points,
                                        const totri_array_t* scan_origin,
                                        const totri_array_t* laser_origin,
                                        const totri_array_t* vg, const float start[3],
                                        const float end[3], float bw, float bo, void* stream_) {
  (void)scan_origin;
  (void)laser_origin;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(check_array(vg, "volume_grad", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_contiguous(vg, "volume_grad"));
  const int64_t B = vg->shape[0];
  int64_t S, L;
  vexh::Pts sp, lp;
  TOTRI_TRY(check_pts(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts(laser_points, "laser_points", B, L, lp));
  TOTRI_TRY(check_array(tg, "transient_grad", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tg, "transient_grad", 0, B));
  TOTRI_TRY(check_dim(tg, "transient_grad", 2, S));
  TOTRI_TRY(check_dim(tg, "transient_grad", 3, L));
  TOTRI_TRY(check_contiguous(tg, "transient_grad"));
  vexh::Geo g{(int)vg->shape[1], (int)vg->shape[2], (int)vg->shape[3], (int)S, (int)L,
              (int)tg->shape[1], start[0], start[1], start[2], end[0], end[1], end[2], bw, bo};
  const int64_t n = numel(vg);
  if (n == 0) return TOTRI_OK;
  TOTRI_KERNEL("volume exhaustive adjoint", stream,
               vexh::adjoint_kernel<<<(unsigned)ceil_div(n, 128), 128, 0, stream>>>(
                   g, (int)B, sp, lp, static_cast<const float*>(tg->data),
                   static_cast<float*>(vg->data)));
  return TOTRI_OK;
}

}  // extern "C"
