// Broad phase of the DEM step: cell hash -> stable LSD radix sort -> cell
// bounds -> slot reorder -> Verlet neighbour lists.
//
// Replaces the reference's serial uniform grid (src/grid.rs:12-87, filled at
// src/simulation.rs:273-276) and its per-particle 27-cell gather. The chain
// runs only on steps that need a rebuild: every kernel here is "gated" on the
// device control block (rebuild requested and no halt), so a captured step
// sequence can contain the whole chain and the host never has to sync to
// decide whether to rebuild.
#include <atomic>

#include "rp_device.cuh"
#include "rp_launch.h"

namespace rp {

int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
  if (dev >= 64) {
    int v = 0;
    return cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 1;
  }
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 1;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

static constexpr uint32_t EMPTY = 0xFFFFFFFFu;
static constexpr int RS_BLOCK = 256;
static constexpr int RS_ITEMS = 8;
static constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;  // keys per block
static constexpr int RS_WARPS = RS_BLOCK / 32;

// A gate is open when it has no control block (diagnostic use) or when a
// rebuild is requested and the chunk has not halted.
__device__ __forceinline__ bool gate_closed(const Ctrl* c) {
  if (!c) return false;
  volatile const Ctrl* v = c;
  return (v->rebuild == 0) || (v->halt != 0);
}

// ------------------------------------------------------------------ hashing
// Fine-grid key of every slot; dead slots go to an extra bucket (fncells)
// that sorts last and is never searched.
__global__ void k_hash_fine(StepParams P, uint32_t* keys, uint32_t* vals) {
  if (gate_closed(P.ctrl)) return;
  const Bank B = P.bank[P.ctrl->bank];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t key;
    if (B.flags[k] & PF_DEAD) key = P.fncells;
    else {
      D4 x = B.xr[k];
      key = fine_cell(P, x.x, x.y, x.z);
    }
    keys[k] = key;
    vals[k] = (uint32_t)k;
  }
}

// Reference-grid key (src/grid.rs:30-40): linear cell or `ncells` when the
// position is outside [0, dims) on any axis (not inserted).
__global__ void k_hash_reference(StepParams P, const D4* xr, int n, uint32_t ncells, uint32_t* keys, uint32_t* vals) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    D4 x = xr[k];
    int32_t c[3];
    ref_coords(P, x.x, x.y, x.z, c);
    uint32_t key = ncells;
    if (c[0] >= 0 && c[1] >= 0 && c[2] >= 0 && c[0] < P.rdims[0] && c[1] < P.rdims[1] && c[2] < P.rdims[2])
      key = (uint32_t)c[0] + (uint32_t)c[1] * (uint32_t)P.rdims[0] +
            (uint32_t)c[2] * (uint32_t)P.rdims[0] * (uint32_t)P.rdims[1];
    keys[k] = key;
    vals[k] = (uint32_t)k;
  }
}

// --------------------------------------------------------------- radix sort
// One 8-bit digit pass: per-block digit histograms, stored digit-major so a
// flat exclusive scan yields every (digit, block) output offset.
__global__ void __launch_bounds__(RS_BLOCK) k_radix_hist(const Ctrl* gate, const uint32_t* keys, uint32_t n, int shift,
                                                          uint32_t* hist, uint32_t nblk) {
  if (gate_closed(gate)) return;
  __shared__ uint32_t s[256];
  for (int d = threadIdx.x; d < 256; d += RS_BLOCK) s[d] = 0;
  __syncthreads();
  uint32_t base = blockIdx.x * RS_TILE;
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    uint32_t idx = base + it * RS_BLOCK + threadIdx.x;
    if (idx < n) {
      uint32_t d = (keys[idx] >> shift) & 255u;
      unsigned peers = __match_any_sync(__activemask(), d);
      int leader = __ffs(peers) - 1;
      if ((int)(threadIdx.x & 31) == leader) atomicAdd(&s[d], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += RS_BLOCK) hist[(size_t)d * nblk + blockIdx.x] = s[d];
}

// Stable scatter: warp w owns keys [base + w*32*ITEMS, +32*ITEMS) and ranks
// them round by round with __match_any_sync, so equal digits keep input order.
__global__ void __launch_bounds__(RS_BLOCK) k_radix_scatter(const Ctrl* gate, const uint32_t* kin, const uint32_t* vin,
                                                             uint32_t* kout, uint32_t* vout, uint32_t n, int shift,
                                                             const uint32_t* offs, uint32_t nblk) {
  if (gate_closed(gate)) return;
  __shared__ uint32_t cnt[RS_WARPS][256];
  __shared__ uint32_t boff[256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_BLOCK) cnt[i >> 8][i & 255] = 0;
  for (int d = threadIdx.x; d < 256; d += RS_BLOCK) boff[d] = offs[(size_t)d * nblk + blockIdx.x];
  __syncthreads();
  uint32_t key[RS_ITEMS], val[RS_ITEMS], rank[RS_ITEMS];
  const uint32_t base = blockIdx.x * RS_TILE + warp * 32 * RS_ITEMS;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    uint32_t idx = base + it * 32 + lane;
    bool valid = idx < n;
    key[it] = valid ? kin[idx] : 0u;
    val[it] = valid ? vin[idx] : 0u;
    uint32_t d = (key[it] >> shift) & 255u;
    unsigned peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 256u + lane);
    uint32_t before = valid ? cnt[warp][d] : 0u;
    rank[it] = before + __popc(peers & lt);
    __syncwarp();
    if (valid && (peers & lt) == 0) cnt[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // exclusive prefix over warps, per digit
  for (int d = threadIdx.x; d < 256; d += RS_BLOCK) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t t = cnt[w][d];
      cnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < RS_ITEMS; ++it) {
    uint32_t idx = base + it * 32 + lane;
    if (idx < n) {
      uint32_t d = (key[it] >> shift) & 255u;
      uint32_t pos = boff[d] + cnt[warp][d] + rank[it];
      kout[pos] = key[it];
      vout[pos] = val[it];
    }
  }
}

// ----------------------------------------------------- device-wide scan (u32)
static constexpr int SC_BLOCK = 256;
static constexpr int SC_ITEMS = 8;
static constexpr int SC_TILE = SC_BLOCK * SC_ITEMS;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t wsum[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nw ? wsum[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < nw) wsum[lane] = wi - w;
    if (lane == nw - 1 && total) *total = wi;
  }
  __syncthreads();
  uint32_t r = inc - v + wsum[warp];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(SC_BLOCK) k_scan_reduce(const Ctrl* gate, const uint32_t* in, uint32_t n,
                                                           uint32_t* part) {
  if (gate_closed(gate)) return;
  uint32_t base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS, s = 0;
#pragma unroll
  for (int i = 0; i < SC_ITEMS; ++i)
    if (base + i < n) s += in[base + i];
  __shared__ uint32_t tot;
  block_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// One block scans the per-tile sums in place, chunk by chunk with a carry.
__global__ void __launch_bounds__(1024) k_scan_top(const Ctrl* gate, uint32_t* part, uint32_t np, uint32_t* total) {
  if (gate_closed(gate)) return;
  __shared__ uint32_t carry_s;
  __shared__ uint32_t tot;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (uint32_t base = 0; base < np; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    uint32_t v = i < np ? part[i] : 0u;
    uint32_t ex = block_exclusive_scan(v, &tot);
    uint32_t c = carry_s;
    if (i < np) part[i] = ex + c;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry_s;
}

__global__ void __launch_bounds__(SC_BLOCK) k_scan_down(const Ctrl* gate, const uint32_t* in, uint32_t* out, uint32_t n,
                                                         const uint32_t* part) {
  if (gate_closed(gate)) return;
  uint32_t base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS;
  uint32_t v[SC_ITEMS], s = 0;
#pragma unroll
  for (int i = 0; i < SC_ITEMS; ++i) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t ex = block_exclusive_scan(s, nullptr) + part[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SC_ITEMS; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
}

void launch_exclusive_scan(const Ctrl* gate, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* part,
                           uint32_t* total, cudaStream_t s) {
  if (n == 0) return;
  uint32_t nb = (n + SC_TILE - 1) / SC_TILE;
  k_scan_reduce<<<nb, SC_BLOCK, 0, s>>>(gate, in, n, part);
  k_scan_top<<<1, 1024, 0, s>>>(gate, part, nb, total);
  k_scan_down<<<nb, SC_BLOCK, 0, s>>>(gate, in, out, n, part);
}

uint32_t scan_parts_needed(uint32_t n) { return (n + SC_TILE - 1) / SC_TILE + 1; }
uint32_t radix_hist_needed(uint32_t n) { return 256u * ((n + RS_TILE - 1) / RS_TILE) + 1; }

// Stable LSD sort of (key, value) pairs on the low `bits` key bits. Input in
// (ka, va); returns 0 when the result is in (ka, va), 1 when in (kb, vb).
int launch_radix_sort(const Ctrl* gate, uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t n, int bits,
                      uint32_t* hist, uint32_t* part, cudaStream_t s) {
  if (n == 0) return 0;
  uint32_t nblk = (n + RS_TILE - 1) / RS_TILE;
  int passes = (bits + 7) / 8;
  if (passes < 1) passes = 1;
  uint32_t *ks = ka, *vs = va, *kd = kb, *vd = vb;
  for (int p = 0; p < passes; ++p) {
    int shift = 8 * p;
    k_radix_hist<<<nblk, RS_BLOCK, 0, s>>>(gate, ks, n, shift, hist, nblk);
    launch_exclusive_scan(gate, hist, hist, 256u * nblk, part, nullptr, s);
    k_radix_scatter<<<nblk, RS_BLOCK, 0, s>>>(gate, ks, vs, kd, vd, n, shift, hist, nblk);
    uint32_t* t = ks; ks = kd; kd = t;
    t = vs; vs = vd; vd = t;
  }
  return (passes & 1) ? 1 : 0;
}

// --------------------------------------------------------------- cell bounds
__global__ void k_fill_u32(const Ctrl* gate, uint32_t* a, uint32_t n, uint32_t v) {
  if (gate_closed(gate)) return;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_cell_bounds(const Ctrl* gate, const uint32_t* skeys, uint32_t n, uint32_t ncells, uint32_t* cstart,
                              uint32_t* cend) {
  if (gate_closed(gate)) return;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    uint32_t key = skeys[k];
    if (key >= ncells) continue;
    if (k == 0 || skeys[k - 1] != key) cstart[key] = k;
    if (k == n - 1 || skeys[k + 1] != key) cend[key] = k + 1;
  }
}

// -------------------------------------------------------------- slot reorder
// Gather every per-slot array of the current bank into the other bank in
// sorted-cell order and remember the build positions for the skin test.
__global__ void k_reorder(StepParams P, const uint32_t* perm) {
  if (gate_closed(P.ctrl)) return;
  const int b = P.ctrl->bank;
  const Bank S = P.bank[b], D = P.bank[b ^ 1];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t o = perm[k];
    D4 x = S.xr[o];
    D.xr[k] = x;
    D.vm[k] = S.vm[o];
    D.wc[k] = S.wc[o];
    D.acc[k] = S.acc[o];
    D.tq[k] = S.tq[o];
    D.xres[k] = S.xres[o];
    D.vres[k] = S.vres[o];
    D.wres[k] = S.wres[o];
    D.flags[k] = S.flags[o];
    D.tag[k] = S.tag[o];
    D.xref[k] = make_float4((float)x.x, (float)x.y, (float)x.z, 0.f);
    D.xf[k] = S.xf[o];
    if (P.ngroups > 1) D.grp[k] = S.grp[o];
  }
}

// --------------------------------------------------------- neighbour lists
// One thread per slot scans the 27 (deduplicated) fine cells around it and
// keeps every other particle within (cutoff + skin), tested in FP32 on the
// FP64 difference with a small relative margin, so the list is a superset of
// every pair the exact FP64 cutoff test can accept before the next rebuild.
// A neighbouring cell farther from the particle than its largest list radius
// (the largest radius as partner) holds no list entry and is skipped.
// Physical mode carries each pair's tangential spring over from the old list.
__global__ void k_build_nlist(StepParams P, const uint32_t* cstart, const uint32_t* cend, const uint32_t* perm,
                              int carry_history) {
  if (gate_closed(P.ctrl)) return;
  const int b = P.ctrl->bank;
  const Bank O = P.bank[b], B = P.bank[b ^ 1];
  const float adh = (P.nmodel == 3 || P.nmodel == 4) ? 1.5f : 1.0f;
  const float skin = (float)P.skin;
  const size_t plane_new = (size_t)P.n * P.cap;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < P.n; k += gridDim.x * blockDim.x) {
    uint32_t* row = B.nbr + (size_t)k * P.cap;
    if (B.flags[k] & PF_DEAD) {
      B.ncnt[k] = 0;
      continue;
    }
    const D4 xi = B.xr[k];
    const float4 xif = B.xf[k];
    const float ri = xif.w;
    const uint32_t gk = P.ngroups > 1 ? B.grp[k] : 0u;  // particles of other groups never interact
    const float Xi = fmaxf(fmaxf(fabsf(xif.x), fabsf(xif.y)), fabsf(xif.z));
    uint32_t cl = fine_cell(P, xi.x, xi.y, xi.z);
    int c[3];
    c[0] = (int)(cl % (uint32_t)P.fdims[0]);
    c[1] = (int)((cl / (uint32_t)P.fdims[0]) % (uint32_t)P.fdims[1]);
    c[2] = (int)(cl / ((uint32_t)P.fdims[0] * (uint32_t)P.fdims[1]));
    // the largest list radius of this particle (any partner: a partner within
    // reach has coordinates below Xi + 2 rb, or within the box bound when it
    // is a periodic image) plus the rounding of an FP32 distance again,
    // grown by 1e-4; the cell gaps keep a thousandth of a cell for the
    // rounding of the lookup
    const float rb = (ri + P.rmaxf) * adh + skin;
    const float Xe = fmaxf(Xi + 2.0f * rb, P.xbound);
    const float rlm = (rb * P.list_scale + 5e-7f * (2.0f * Xe + P.lmax + rb)) * 1.0001f;
    const double pq[3] = {xi.x, xi.y, xi.z};
    int off[3][3], no[3];
    float gap[3][3];  // distance from the particle to each listed cell's slab (0: its own)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      no[a] = 0;
      // position within its cell along the axis (the wrap as in fine_cell)
      double q = pq[a] - P.fmin[a];
      if (P.periodic[a]) q = q - floor(q * P.binv[a]) * P.bsize[a];
      const float u = (float)(q - (double)c[a] * P.fcell[a]);
      const float slack = 1e-3f * P.fcellf[a];
      if (P.fdims[a] >= 3) {
        for (int d = -1; d <= 1; ++d) {
          int qq = c[a] + d;
          if (P.periodic[a]) {
            if (qq < 0) qq += P.fdims[a];
            else if (qq >= P.fdims[a]) qq -= P.fdims[a];
          }
          if (qq >= 0 && qq < P.fdims[a]) {
            const float g = d < 0 ? u : (d > 0 ? P.fcellf[a] - u : 0.0f);
            gap[a][no[a]] = fmaxf(g - slack, 0.0f);
            off[a][no[a]++] = qq;
          }
        }
      } else {
        for (int qq = 0; qq < P.fdims[a]; ++qq) {
          gap[a][no[a]] = 0.0f;
          off[a][no[a]++] = qq;
        }
      }
    }
    uint32_t cnt = 0;
    unsigned long long hm = 0ull;  // springs carried over with a value other than +0
    const uint32_t ok = carry_history ? perm[k] : 0u;
    const uint32_t ocnt = carry_history ? O.ncnt[ok] : 0u;
    const uint32_t* orow = O.nbr + (size_t)ok * P.cap;
    const size_t plane_old = plane_new;
    for (int zz = 0; zz < no[2]; ++zz)
      for (int yy = 0; yy < no[1]; ++yy)
        for (int xx = 0; xx < no[0]; ++xx) {
          if (gap[0][xx] * gap[0][xx] + gap[1][yy] * gap[1][yy] + gap[2][zz] * gap[2][zz] > rlm * rlm) continue;
          uint32_t cell = (uint32_t)off[0][xx] + (uint32_t)P.fdims[0] * ((uint32_t)off[1][yy] + (uint32_t)P.fdims[1] * (uint32_t)off[2][zz]);
          uint32_t s = cstart[cell];
          if (s == EMPTY) continue;
          uint32_t e = cend[cell];
          for (uint32_t j = s; j < e; ++j) {
            if ((int)j == k) continue;
            if (P.ngroups > 1 && B.grp[j] != gk) continue;
            // FP32 on the position mirror: each difference is within
            // 2^-24 (2X + |d| + L) of the exact one, so growing the radius by
            // 2.5e-7 (2X + L) + a relative 1e-5 keeps the list a superset
            const float4 xj = B.xf[j];
            float fx = xif.x - xj.x, fy = xif.y - xj.y, fz = xif.z - xj.z;
            // minimum image; where |f| < 0.49 L the image is the pair itself
            if (P.periodic[0] && fabsf(fx * P.binvf[0]) > 0.49f) fx -= P.bsizef[0] * rintf(fx / P.bsizef[0]);
            if (P.periodic[1] && fabsf(fy * P.binvf[1]) > 0.49f) fy -= P.bsizef[1] * rintf(fy / P.bsizef[1]);
            if (P.periodic[2] && fabsf(fz * P.binvf[2]) > 0.49f) fz -= P.bsizef[2] * rintf(fz / P.bsizef[2]);
            float d2 = fx * fx + fy * fy + fz * fz;
            const float X = fmaxf(Xi, fmaxf(fmaxf(fabsf(xj.x), fabsf(xj.y)), fabsf(xj.z)));
            float rl = (ri + xj.w) * adh + skin;
            rl = rl * P.list_scale + 2.5e-7f * (2.0f * X + P.lmax);
            if (d2 < rl * rl) {
              if (cnt < (uint32_t)P.cap) {
                row[cnt] = j;
                if (carry_history) {
                  double h0 = 0.0, h1 = 0.0, h2 = 0.0;
                  uint32_t oj = perm[j];
                  for (uint32_t q = 0; q < ocnt; ++q)
                    if (orow[q] == oj) {
                      size_t oi = (size_t)ok * P.cap + q;
                      h0 = O.hist[oi];
                      h1 = O.hist[plane_old + oi];
                      h2 = O.hist[2 * plane_old + oi];
                      break;
                    }
                  size_t ni = (size_t)k * P.cap + cnt;
                  B.hist[ni] = h0;
                  B.hist[plane_new + ni] = h1;
                  B.hist[2 * plane_new + ni] = h2;
                  if (cnt < 64 && (__double_as_longlong(h0) | __double_as_longlong(h1) | __double_as_longlong(h2)))
                    hm |= 1ull << cnt;
                }
              }
              ++cnt;
            }
          }
        }
    B.ncnt[k] = cnt < (uint32_t)P.cap ? cnt : (uint32_t)P.cap;
    if (carry_history) B.hmask[k] = hm;
    atomicMax(&P.ctrl->max_count, cnt);
    if (cnt > (uint32_t)P.cap) atomicOr(&P.ctrl->halt, HALT_LISTS);
  }
}

__global__ void k_rebuild_finish(StepParams P) {
  Ctrl* c = P.ctrl;
  if (c->rebuild == 0 || c->halt != 0) return;
  c->bank ^= 1;
  c->rebuild = 0;
  c->rebuilds += 1;
}

// Old-list slots are indexed by old slot numbers, so the history lookup in
// k_build_nlist needs perm (new slot -> old slot) for both ends of a pair.
int launch_rebuild(const StepParams& P, const RebuildBufs& R, cudaStream_t s) {
  const Ctrl* g = P.ctrl;
  const int passes = (R.key_bits + 7) / 8 < 1 ? 1 : (R.key_bits + 7) / 8;
  const int nb = grid_for(P.n, 256);
  k_hash_fine<<<nb, 256, 0, s>>>(P, R.ka, R.va);
  int which = launch_radix_sort(g, R.ka, R.va, R.kb, R.vb, (uint32_t)P.n, R.key_bits, R.hist, R.part, s);
  uint32_t* sk = which ? R.kb : R.ka;
  uint32_t* sv = which ? R.vb : R.va;
  k_fill_u32<<<grid_for(P.fncells, 256), 256, 0, s>>>(g, R.cstart, P.fncells, EMPTY);
  k_cell_bounds<<<nb, 256, 0, s>>>(g, sk, (uint32_t)P.n, P.fncells, R.cstart, R.cend);
  k_reorder<<<nb, 256, 0, s>>>(P, sv);
  k_build_nlist<<<grid_for(P.n, 128), 128, 0, s>>>(P, R.cstart, R.cend, sv, R.carry_history);
  const int ko = launch_accum_order(P, s);
  k_rebuild_finish<<<1, 1, 0, s>>>(P);
  return 1 + 5 * passes + 5 + ko;
}

// Diagnostic: the reference grid's key per slot (written to kraw) and the
// stable cell order (the sorted values).
int launch_reference_grid(const StepParams& P, const D4* xr, int n, uint32_t ncells, int key_bits, uint32_t* kraw,
                          uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t* hist, uint32_t* part,
                          cudaStream_t s) {
  k_hash_reference<<<grid_for(n, 256), 256, 0, s>>>(P, xr, n, ncells, ka, va);
  cudaMemcpyAsync(kraw, ka, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  return launch_radix_sort(nullptr, ka, va, kb, vb, (uint32_t)n, key_bits, hist, part, s);
}

}  // namespace rp
