// LBVH construction for a batch of meshes.
//
// Replaces the per-call OptiX acceleration-structure build of the reference
// (TriangleGas::Update, src/common/optix.cu:33-99, with the face compaction of
// FacesTensor2Buffer :18-30 and the thrust::find count :55-58). Every stage
// runs on the device for all batch items at once with no host round trip:
//   1. init      face count = F, bounds reset
//   2. faces     first face holding an index outside [0, V) ends the list
//   3. bounds    centroid AABB (Morton frame) and coordinate scale
//   4. morton    30-bit Morton code of each centroid
//   5. sort      stable LSD radix sort of (code, face), one CTA per mesh
//   6. records   sorted TriRec / ShadeRec
//   7. hierarchy Karras 2012 internal nodes, parent links
//   8. refit     bottom-up boxes (second arrival at a node merges its children)
#include "mesh.cuh"
#include "tune.cuh"

namespace totri {
namespace mesh {

namespace {

constexpr int kSortThreads = 1024;
constexpr int kSortBits = 10;
constexpr int kSortDigits = 1 << kSortBits;
constexpr int kSortUnroll = 4;  // batches of 32 keys loaded ahead per warp

__global__ void init_kernel(Scene sc, int F) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < sc.F) sc.counter[(size_t)b * sc.F + i] = 0;
  if (i == 0) {
    Meta& m = sc.meta[b];
    m.n = F;
    m.term_neg = 0;
    m.scale = 0.f;
    m.delta = 0.f;
    for (int a = 0; a < 3; ++a) {
      m.cmin[a] = ford(3.0e38f);
      m.cmax[a] = ford(-3.0e38f);
    }
  }
  if (b == 0 && i == 0 && blockIdx.x == 0) {
    // status word is cleared by the host with a memset
  }
}

__global__ void faces_kernel(Scene sc, BuildInputs in) {
  const int b = blockIdx.y;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= in.F) return;
  bool bad = false;
  for (int k = 0; k < 3; ++k) {
    const int64_t v = in.faces.at(b, f, k);
    bad |= (v < 0 || v >= in.V);
  }
  if (bad) atomicMin(&sc.meta[b].n, f);
}

__device__ __forceinline__ fv3 load_vert(const BuildInputs& in, int b, int64_t v) {
  return mkv(in.verts.at(b, v, 0), in.verts.at(b, v, 1), in.verts.at(b, v, 2));
}

__device__ __forceinline__ void face_verts(const BuildInputs& in, int b, int f, fv3 v[3],
                                           int64_t idx[3]) {
  for (int k = 0; k < 3; ++k) {
    idx[k] = in.faces.at(b, f, k);
    v[k] = load_vert(in, b, idx[k]);
  }
}

__global__ void bounds_kernel(Scene sc, BuildInputs in) {
  const int b = blockIdx.y;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  float scale = 0.f;
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  if (f < n) {
    fv3 v[3];
    int64_t idx[3];
    face_verts(in, b, f, v, idx);
    for (int k = 0; k < 3; ++k) {
      scale = fmaxf(scale, fmaxf(fabsf(v[k].x), fmaxf(fabsf(v[k].y), fabsf(v[k].z))));
    }
    const fv3 c = xcentroid(v[0], v[1], v[2]);
    const float cc[3] = {c.x, c.y, c.z};
    for (int a = 0; a < 3; ++a) {
      if (cc[a] == cc[a]) {
        lo[a] = cc[a];
        hi[a] = cc[a];
      }
    }
  } else if (f == n && n < in.F) {
    // The terminating face: flag it when no index is negative (index >= V).
    bool neg = false;
    for (int k = 0; k < 3; ++k) neg |= in.faces.at(b, f, k) < 0;
    if (!neg) atomicOr(sc.status, kStatusFaceIndexRange);
  }
  // warp reduction, one atomic per warp and quantity
  for (int off = 16; off > 0; off >>= 1) {
    scale = fmaxf(scale, __shfl_xor_sync(0xffffffffu, scale, off));
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
      hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
    }
  }
  if ((threadIdx.x & 31) == 0 && blockIdx.x * blockDim.x + (threadIdx.x & ~31) < n) {
    Meta& m = sc.meta[b];
    atomicMax(reinterpret_cast<int*>(&m.scale), __float_as_int(scale));
    for (int a = 0; a < 3; ++a) {
      atomicMin(&m.cmin[a], ford(lo[a]));
      atomicMax(&m.cmax[a], ford(hi[a]));
    }
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void morton_kernel(Scene sc, BuildInputs in) {
  const int b = blockIdx.y;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  if (f >= n) return;
  fv3 v[3];
  int64_t idx[3];
  face_verts(in, b, f, v, idx);
  const fv3 c = xcentroid(v[0], v[1], v[2]);
  const Meta& m = sc.meta[b];
  const float cc[3] = {c.x, c.y, c.z};
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) {
    const float lo = iord(m.cmin[a]), hi = iord(m.cmax[a]);
    const float ext = hi - lo;
    float u = ext > 0.f ? (cc[a] - lo) / ext : 0.f;
    u = fminf(fmaxf(u, 0.f), 1.f);
    if (!(u == u)) u = 0.f;
    q[a] = (uint32_t)fminf(u * 1024.f, 1023.f);
  }
  const size_t base = (size_t)b * 2 * sc.F;
  sc.keys[base + f] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  sc.vals[base + f] = (uint32_t)f;
}

// One-CTA stable LSD radix sort of n 30-bit keys with their values: three
// 10-bit passes k0/v0 -> k1/v1 -> k0/v0 -> k1/v1, so the sorted pairs end in
// k1/v1. Warp w owns the w-th of 32 contiguous chunks of the input. A pass
// counts each warp's digits (wcount[w][digit]), turns the counts into each
// warp's first output position per digit with one scan over the warps and one
// over the digits, and then lets every warp scatter its chunk in order, 32
// keys at a time, ranking equal digits within the batch with
// __match_any_sync. Warps own ordered ranges and keep their batches in order,
// so the sort is stable.
__device__ void cta_radix_sort30(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, int n,
                                 uint32_t* smem) {
  uint32_t* wcount = smem;                     // [32][1024] per-warp digit count, then cursor
  uint32_t* offset = smem + 32 * kSortDigits;  // [1024] first position of each digit
  uint32_t* total = offset + kSortDigits;      // [1024] digit totals; [32] scan partials
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const int chunk = (((n + 31) / 32) + 31) & ~31;
  const int lo = min(n, warp * chunk), hi = min(n, lo + chunk);
  uint32_t* mine = wcount + warp * kSortDigits;
  for (int pass = 0; pass < 3; ++pass) {
    const int shift = pass * kSortBits;
    const uint32_t* ksrc = (pass & 1) ? k1 : k0;
    const uint32_t* vsrc = (pass & 1) ? v1 : v0;
    uint32_t* kdst = (pass & 1) ? k0 : k1;
    uint32_t* vdst = (pass & 1) ? v0 : v1;
    for (int d = lane; d < kSortDigits; d += 32) mine[d] = 0;
    __syncwarp();
    for (int base = lo; base < hi; base += 32 * kSortUnroll) {
      uint32_t key[kSortUnroll];  // loads of kSortUnroll batches in flight together
#pragma unroll
      for (int u = 0; u < kSortUnroll; ++u) {
        const int i = base + 32 * u + lane;
        key[u] = i < hi ? ksrc[i] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kSortUnroll; ++u) {
        const bool valid = base + 32 * u + lane < hi;
        const uint32_t digit = valid ? ((key[u] >> shift) & (kSortDigits - 1)) : kSortDigits;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        if (valid && lane == __ffs(peers) - 1) mine[digit] += __popc(peers);
        __syncwarp();
      }
    }
    __syncthreads();
    {  // digit tid: exclusive prefix over the warps, then over the digits
      uint32_t run = 0;
      for (int w = 0; w < 32; ++w) {
        const uint32_t c = wcount[w * kSortDigits + tid];
        wcount[w * kSortDigits + tid] = run;
        run += c;
      }
      uint32_t incl = run;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (lane == 31) total[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const uint32_t w = total[lane];
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
          if (lane >= o) wi += y;
        }
        total[lane] = wi - w;
      }
      __syncthreads();
      offset[tid] = total[warp] + incl - run;
      __syncthreads();
    }
    for (int base = lo; base < hi; base += 32 * kSortUnroll) {
      uint32_t key[kSortUnroll], val[kSortUnroll];
#pragma unroll
      for (int u = 0; u < kSortUnroll; ++u) {
        const int i = base + 32 * u + lane;
        key[u] = i < hi ? ksrc[i] : 0u;
        val[u] = i < hi ? vsrc[i] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kSortUnroll; ++u) {
        const bool valid = base + 32 * u + lane < hi;
        const uint32_t digit = valid ? ((key[u] >> shift) & (kSortDigits - 1)) : kSortDigits;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t cur = 0;
        if (valid) {
          cur = mine[digit];
          const uint32_t pos = offset[digit] + cur + __popc(peers & lt);
          kdst[pos] = key[u];
          vdst[pos] = val[u];
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) mine[digit] = cur + __popc(peers);
        __syncwarp();
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kSortThreads) sort_kernel(Scene sc) {
  extern __shared__ uint32_t smem[];
  const int b = blockIdx.x;
  uint32_t* k0 = sc.keys + (size_t)b * 2 * sc.F;
  uint32_t* v0 = sc.vals + (size_t)b * 2 * sc.F;
  cta_radix_sort30(k0, v0, k0 + sc.F, v0 + sc.F, sc.meta[b].n, smem);
}

// Morton order of P wall points, one CTA per batch item: bounding box, 30-bit
// codes over it, radix sort. scr is [4][B][P] (keys, values, keys, values);
// the permutation (point indices in Morton order) ends in the fourth quarter,
// and the first quarter is then set to -1: the visibility kernel keeps each
// point's last occluder there (by Morton position of the point).
__global__ void __launch_bounds__(kSortThreads) point_order_kernel(View3f pts, int P, int B,
                                                                  uint32_t* scr) {
  extern __shared__ uint32_t smem[];
  __shared__ int box[6];
  const int b = blockIdx.x;
  const size_t BP = (size_t)B * P;
  uint32_t* k0 = scr + (size_t)b * P;
  uint32_t* v0 = scr + BP + (size_t)b * P;
  uint32_t* k1 = scr + 2 * BP + (size_t)b * P;
  uint32_t* v1 = scr + 3 * BP + (size_t)b * P;
  if (threadIdx.x < 3) {
    box[threadIdx.x] = ford(3.0e38f);
    box[3 + threadIdx.x] = ford(-3.0e38f);
  }
  __syncthreads();
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    for (int a = 0; a < 3; ++a) {
      const float c = pts.at(b, i, a);
      lo[a] = fminf(lo[a], c);
      hi[a] = fmaxf(hi[a], c);
    }
  for (int a = 0; a < 3; ++a) {
    atomicMin(&box[a], ford(lo[a]));
    atomicMax(&box[3 + a], ford(hi[a]));
  }
  __syncthreads();
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
      const float l = iord(box[a]), ext = iord(box[3 + a]) - l;
      float u = ext > 0.f ? (pts.at(b, i, a) - l) / ext : 0.f;
      u = fminf(fmaxf(u, 0.f), 1.f);
      if (!(u == u)) u = 0.f;
      q[a] = (uint32_t)fminf(u * 1024.f, 1023.f);
    }
    k0[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    v0[i] = (uint32_t)i;
  }
  __syncthreads();
  cta_radix_sort30(k0, v0, k1, v1, P, smem);
  __syncthreads();
  for (int i = threadIdx.x; i < P; i += blockDim.x) k0[i] = ~0u;
}

__global__ void records_kernel(Scene sc, BuildInputs in) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const Meta& m = sc.meta[b];
  const int n = m.n;
  if (k >= n) return;
  int f = (int)sc.vals[(size_t)b * 2 * sc.F + (size_t)sc.sorted_buf * sc.F + k];
  if (!TOTRI_INDEX_OK((unsigned)f < (unsigned)in.F, sc.status)) f = 0;
  fv3 v[3];
  int64_t idx[3];
  face_verts(in, b, f, v, idx);
  const float delta = ldexpf(m.scale, -12);
  const fv3 e1 = xsub3(v[1], v[0]), e2 = xsub3(v[2], v[0]);
  const float lox = xsub(fminf(fminf(v[0].x, v[1].x), v[2].x), delta);
  const float loy = xsub(fminf(fminf(v[0].y, v[1].y), v[2].y), delta);
  const float loz = xsub(fminf(fminf(v[0].z, v[1].z), v[2].z), delta);
  const float hix = xadd(fmaxf(fmaxf(v[0].x, v[1].x), v[2].x), delta);
  const float hiy = xadd(fmaxf(fmaxf(v[0].y, v[1].y), v[2].y), delta);
  const float hiz = xadd(fmaxf(fmaxf(v[0].z, v[1].z), v[2].z), delta);
  float4* t = sc.tri + ((size_t)b * sc.F + k) * 4;
  t[0] = make_float4(v[0].x, v[0].y, v[0].z, e1.x);
  t[1] = make_float4(e1.y, e1.z, e2.x, e2.y);
  t[2] = make_float4(e2.z, lox, loy, loz);
  t[3] = make_float4(hix, hiy, hiz, __int_as_float(f));
  float rho = 1.f;
  if (in.M > 0) {
    const float third = 1.f / 3.f;
    rho = third * ((in.material.at(b, idx[0], 0) + in.material.at(b, idx[1], 0)) +
                   in.material.at(b, idx[2], 0));
  }
  const fv3 c = xcentroid(v[0], v[1], v[2]);
  float4* s = sc.shade + ((size_t)b * sc.F + k) * 4;
  s[0] = make_float4(v[0].x, v[0].y, v[0].z, rho);
  s[1] = make_float4(v[1].x, v[1].y, v[1].z, __int_as_float((int)idx[0]));
  s[2] = make_float4(v[2].x, v[2].y, v[2].z, __int_as_float((int)idx[1]));
  s[3] = make_float4(c.x, c.y, c.z, __int_as_float((int)idx[2]));
  if (k == 0) sc.meta[b].delta = delta;
}

__device__ __forceinline__ int kdelta(const uint32_t* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = keys[i], c = keys[j];
  if (a == c) return 32 + __clz((uint32_t)(i ^ j));
  return __clz(a ^ c);
}

__global__ void hierarchy_kernel(Scene sc) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  if (i >= n - 1) return;
  const uint32_t* keys = sc.keys + (size_t)b * 2 * sc.F + (size_t)sc.sorted_buf * sc.F;
  const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(keys, n, i, i - d);
  int lmax = 2;
  while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = kdelta(keys, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  const int left = (lo == gamma) ? ~gamma : gamma;
  const int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  float4* nd = sc.nodes + ((size_t)b * sc.F + i) * 4;
  nd[3] = make_float4(__int_as_float(left), __int_as_float(right), 0.f, 0.f);
  const size_t base = (size_t)b * sc.F;
  if (left < 0) sc.lparent[base + ~left] = i; else sc.iparent[base + left] = i;
  if (right < 0) sc.lparent[base + ~right] = i; else sc.iparent[base + right] = i;
  if (i == 0) sc.iparent[base] = -1;
}

__global__ void refit_kernel(Scene sc) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  if (k >= n || n < 2) return;
  const float delta = sc.meta[b].delta;
  const float4* t = sc.tri + ((size_t)b * sc.F + k) * 4;
  const float4 t2 = t[2], t3 = t[3];
  // BVH leaf box: hit-point box grown by another delta.
  float lo[3] = {t2.y - delta, t2.z - delta, t2.w - delta};
  float hi[3] = {t3.x + delta, t3.y + delta, t3.z + delta};
  const size_t base = (size_t)b * sc.F;
  int child = ~k;
  int node = sc.lparent[base + k];
  while (node >= 0) {
    float* nd = reinterpret_cast<float*>(sc.nodes + (base + node) * 4);
    const int c0 = __float_as_int(nd[12]);
    const int side = c0 == child ? 0 : 1;
    for (int a = 0; a < 3; ++a) {
      nd[node_plane(side, 0, a)] = lo[a];
      nd[node_plane(side, 1, a)] = hi[a];
    }
    __threadfence();
    if (atomicAdd(&sc.counter[base + node], 1) == 0) return;
    __threadfence();
    const volatile float* vn = nd;
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(vn[node_plane(0, 0, a)], vn[node_plane(1, 0, a)]);
      hi[a] = fmaxf(vn[node_plane(0, 1, a)], vn[node_plane(1, 1, a)]);
    }
    child = node;
    node = sc.iparent[base + node];
  }
}

}  // namespace

// 4-wide node records at the even-depth binary nodes: a binary node's child
// boxes are replaced by its grandchildren's (a leaf child keeps its own box and
// slot), read after the refit has finished every box. Slots 0 and 1 are always
// filled; an unused slot carries the code kWideEmpty (traversals skip it).
__global__ void widen_kernel(Scene sc) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  if (i >= n - 1) return;
  const size_t base = (size_t)b * sc.F;
  int depth = 0;
  for (int q = sc.iparent[base + i]; q >= 0 && depth < 4096; q = sc.iparent[base + q]) ++depth;
  if (depth & 1) return;
  const float* nd = reinterpret_cast<const float*>(sc.nodes + (base + i) * 4);
  float box[6][4];
  int code[4] = {kWideEmpty, kWideEmpty, kWideEmpty, kWideEmpty};
  for (int a = 0; a < 6; ++a)
    for (int m = 0; m < 4; ++m) box[a][m] = 0.f;
  int m = 0;
  for (int side = 0; side < 2; ++side) {
    const int c = __float_as_int(nd[12 + side]);
    if (c < 0 || c >= n - 1) {  // leaf (or malformed link: walked and flagged later)
      for (int a = 0; a < 6; ++a) box[a][m] = nd[node_plane(side, a / 3, a % 3)];
      code[m++] = c;
    } else {
      const float* cn = reinterpret_cast<const float*>(sc.nodes + (base + c) * 4);
      for (int g = 0; g < 2; ++g) {
        for (int a = 0; a < 6; ++a) box[a][m] = cn[node_plane(g, a / 3, a % 3)];
        code[m++] = __float_as_int(cn[12 + g]);
      }
    }
  }
  float4* w = sc.wide + (base + i) * 8;
  for (int a = 0; a < 6; ++a) w[a] = make_float4(box[a][0], box[a][1], box[a][2], box[a][3]);
  w[6] = make_float4(__int_as_float(code[0]), __int_as_float(code[1]), __int_as_float(code[2]),
                     __int_as_float(code[3]));
  w[7] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Edge adjacency of the valid faces, in Morton positions. Each face inserts
// its three edges (the unordered pair of vertex indices) into an
// open-addressing hash table of 4 F slots per item; a slot keeps the first two
// faces that hold its edge. Adjacency only steers the surface walk that seeds
// the visibility query with likely occluders: it never decides a mask bit, so
// non-manifold edges (a third face is left out), seams with duplicated
// vertices (no neighbour) and degenerate faces cost speed, not exactness.
constexpr unsigned long long kEdgeEmpty = ~0ull;

__device__ __forceinline__ unsigned long long edge_key(uint32_t a, uint32_t c) {
  return a < c ? ((unsigned long long)a << 32) | c : ((unsigned long long)c << 32) | a;
}

__device__ __forceinline__ int edge_slot(unsigned long long key, int cap) {
  return (int)(((key * 0x9E3779B97F4A7C15ull) >> 32) % (unsigned long long)cap);
}

__device__ __forceinline__ void face_vertex_ids(const Scene& sc, int b, int k, uint32_t vi[3]) {
  const float4* s = sc.shade + ((size_t)b * sc.F + k) * 4;
  vi[0] = (uint32_t)__float_as_int(s[1].w);
  vi[1] = (uint32_t)__float_as_int(s[2].w);
  vi[2] = (uint32_t)__float_as_int(s[3].w);
}

__global__ void edge_insert_kernel(Scene sc) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sc.meta[b].n) return;
  uint32_t vi[3];
  face_vertex_ids(sc, b, k, vi);
  unsigned long long* keys = sc.ekeys + (size_t)b * sc.ecap;
  int2* vals = sc.evals + (size_t)b * sc.ecap;
  for (int e = 0; e < 3; ++e) {
    const uint32_t a = vi[(e + 1) % 3], c = vi[(e + 2) % 3];
    if (a == c) continue;
    const unsigned long long key = edge_key(a, c);
    int h = edge_slot(key, sc.ecap);
    for (int it = 0; it < sc.ecap; ++it) {  // 3 n <= 3 F keys in 4 F slots: a slot is found
      const unsigned long long prev = atomicCAS(&keys[h], kEdgeEmpty, key);
      if (prev == kEdgeEmpty || prev == key) {
        if (atomicCAS(&vals[h].x, -1, k) != -1) atomicCAS(&vals[h].y, -1, k);
        break;
      }
      h = h + 1 == sc.ecap ? 0 : h + 1;
    }
  }
}

__global__ void edge_link_kernel(Scene sc) {
  const int b = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sc.meta[b].n) return;
  uint32_t vi[3];
  face_vertex_ids(sc, b, k, vi);
  const unsigned long long* keys = sc.ekeys + (size_t)b * sc.ecap;
  const int2* vals = sc.evals + (size_t)b * sc.ecap;
  int nb[3];
  for (int e = 0; e < 3; ++e) {
    nb[e] = -1;
    const uint32_t a = vi[(e + 1) % 3], c = vi[(e + 2) % 3];
    if (a == c) continue;
    const unsigned long long key = edge_key(a, c);
    int h = edge_slot(key, sc.ecap);
    for (int it = 0; it < sc.ecap; ++it) {
      const unsigned long long kk = keys[h];
      if (kk == key) {
        const int2 v = vals[h];
        nb[e] = v.x == k ? v.y : v.x;
        break;
      }
      if (kk == kEdgeEmpty) break;
      h = h + 1 == sc.ecap ? 0 : h + 1;
    }
    if (nb[e] == k) nb[e] = -1;
  }
  sc.adj[(size_t)b * sc.F + k] = make_int4(nb[0], nb[1], nb[2], 0);
}

int launch_point_order(const Scene& sc, const View3f& pts, int P, cudaStream_t stream) {
  const size_t smem = sizeof(uint32_t) * (32 * kSortDigits + 2 * kSortDigits);
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(point_order_kernel), smem));
  TOTRI_KERNEL("mesh point order", stream,
               point_order_kernel<<<sc.B, kSortThreads, smem, stream>>>(pts, P, sc.B,
                                                                         sc.pscratch));
  return TOTRI_OK;
}

int build_scene(const Scene& sc, const BuildInputs& in, cudaStream_t stream) {
  const int B = sc.B;
  const dim3 blk(256);
  const dim3 gridF((unsigned)ceil_div(sc.F, 256), (unsigned)B);
  TOTRI_CUDA(cudaMemsetAsync(sc.status, 0, sizeof(uint32_t), stream));
  TOTRI_KERNEL("mesh init", stream, init_kernel<<<gridF, blk, 0, stream>>>(sc, in.F));
  if (in.F > 0) {
    TOTRI_KERNEL("mesh faces", stream, faces_kernel<<<gridF, blk, 0, stream>>>(sc, in));
    TOTRI_KERNEL("mesh bounds", stream, bounds_kernel<<<gridF, blk, 0, stream>>>(sc, in));
    TOTRI_KERNEL("mesh morton", stream, morton_kernel<<<gridF, blk, 0, stream>>>(sc, in));
    const size_t smem = sizeof(uint32_t) * (32 * kSortDigits + 2 * kSortDigits);
    TOTRI_CUDA(tune::ensure_dynamic_smem(
        reinterpret_cast<const void*>(sort_kernel), smem));
    TOTRI_KERNEL("mesh sort", stream, sort_kernel<<<B, kSortThreads, smem, stream>>>(sc));
    TOTRI_KERNEL("mesh records", stream, records_kernel<<<gridF, blk, 0, stream>>>(sc, in));
    TOTRI_CUDA(cudaMemsetAsync(sc.ekeys, 0xff, sizeof(unsigned long long) * B * sc.ecap, stream));
    TOTRI_CUDA(cudaMemsetAsync(sc.evals, 0xff, sizeof(int2) * B * sc.ecap, stream));
    TOTRI_KERNEL("mesh edges", stream, edge_insert_kernel<<<gridF, blk, 0, stream>>>(sc));
    TOTRI_KERNEL("mesh edges", stream, edge_link_kernel<<<gridF, blk, 0, stream>>>(sc));
    TOTRI_KERNEL("mesh hierarchy", stream, hierarchy_kernel<<<gridF, blk, 0, stream>>>(sc));
    TOTRI_KERNEL("mesh refit", stream, refit_kernel<<<gridF, blk, 0, stream>>>(sc));
    TOTRI_KERNEL("mesh widen", stream, widen_kernel<<<gridF, blk, 0, stream>>>(sc));
  }
  return TOTRI_OK;
}

}  // namespace mesh
}  // namespace totri
