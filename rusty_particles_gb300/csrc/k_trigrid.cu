// The triangle grid of the wall contacts, built on the device.
//
// The reference tests every triangle of every mesh against every particle
// (src/simulation.rs:464-523). The step instead looks up the triangles listed
// in the uniform-grid cell of a particle's centre, in mesh order, so the
// contacts and their summation order are the reference's. A triangle is
// listed in every cell of its bounding box grown by the largest radius whose
// centre lies within half a cell diagonal plus that growth of the triangle
// (point-triangle distance, Ericson, Real-Time Collision Detection, 2005,
// 5.1.5): a centre that lands in such a cell and lies within the largest
// radius of the triangle is within that distance of the cell's centre.
//
// The host keeps the O(T) set-up next to the mesh it owns (grown boxes, the
// cell size, the per-triangle candidate counts); the device computes the
// per-triangle records, tests every (triangle, cell) candidate and groups the
// survivors by cell with a stable radix sort, so each cell lists its
// triangles in mesh order. Compiled without contraction (-fmad=false): every
// value rounds as the host's double arithmetic would.
#include <algorithm>
#include <cmath>

#include "rp_device.cuh"
#include "rp_launch.h"

namespace rp {

// Per-triangle constants of src/mesh.rs:45-62 and the FP32 pretest planes.
__global__ void k_tri_records(const float* __restrict__ v, const float* __restrict__ nrm,
                              const uint32_t* __restrict__ grp, const uint32_t* __restrict__ mot, int T,
                              TriRec* __restrict__ recs) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
    const float* q = v + 9 * (size_t)t;
    const double v0[3] = {q[0], q[1], q[2]}, v1[3] = {q[3], q[4], q[5]}, v2[3] = {q[6], q[7], q[8]};
    TriRec r;
    for (int k = 0; k < 3; ++k) {
      r.v0[k] = v0[k];
      r.e0[k] = v1[k] - v0[k];
      r.e1[k] = v2[k] - v0[k];
      r.n[k] = nrm[3 * (size_t)t + k];
    }
    r.a = r.e0[0] * r.e0[0] + r.e0[1] * r.e0[1] + r.e0[2] * r.e0[2];
    r.b = r.e0[0] * r.e1[0] + r.e0[1] * r.e1[1] + r.e0[2] * r.e1[2];
    r.c = r.e1[0] * r.e1[0] + r.e1[1] * r.e1[1] + r.e1[2] * r.e1[2];
    r.det = r.a * r.c - r.b * r.b;
    r.denom = r.a - 2.0 * r.b + r.c;
    r.group = grp[t];
    r.motion = mot[t];
    double cx = r.e0[1] * r.e1[2] - r.e0[2] * r.e1[1], cy = r.e0[2] * r.e1[0] - r.e0[0] * r.e1[2],
           cz = r.e0[0] * r.e1[1] - r.e0[1] * r.e1[0];
    const double l = sqrt(cx * cx + cy * cy + cz * cz);
    for (int e = 0; e < 3; ++e) r.edge[e] = make_float4(0.f, 0.f, 0.f, 1e30f);  // never rejects
    if (l > 0.0 && isfinite(l)) {
      cx /= l;
      cy /= l;
      cz /= l;
      r.plane = make_float4((float)cx, (float)cy, (float)cz, (float)(cx * v0[0] + cy * v0[1] + cz * v0[2]));
      // in-plane unit normals of the edges, pointing away from the triangle
      const double* vv[3] = {v0, v1, v2};
      for (int e = 0; e < 3; ++e) {
        const double *p = vv[e], *q2 = vv[(e + 1) % 3], *o = vv[(e + 2) % 3];
        const double d[3] = {q2[0] - p[0], q2[1] - p[1], q2[2] - p[2]};
        double m[3] = {d[1] * cz - d[2] * cy, d[2] * cx - d[0] * cz, d[0] * cy - d[1] * cx};
        const double ml = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        if (!(ml > 0.0) || !isfinite(ml)) continue;
        for (int k = 0; k < 3; ++k) m[k] /= ml;
        if (m[0] * (o[0] - p[0]) + m[1] * (o[1] - p[1]) + m[2] * (o[2] - p[2]) > 0.0)
          for (int k = 0; k < 3; ++k) m[k] = -m[k];
        r.edge[e] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)(m[0] * p[0] + m[1] * p[1] + m[2] * p[2]));
      }
    } else {
      r.plane = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    double vm = 0.0;
    for (int k = 0; k < 3; ++k) vm = fmax(vm, fmax(fabs(v0[k]), fmax(fabs(v1[k]), fabs(v2[k]))));
    r.bound = make_float4((float)vm, 0.f, 0.f, 0.f);
    recs[t] = r;
  }
}

// Squared distance from p to the triangle (a, b, c): the closest point by its
// Voronoi region (Ericson 2005, 5.1.5).
__device__ double point_triangle_dist2(const double p[3], const double a[3], const double b[3], const double c[3]) {
  double ab[3], ac[3], ap[3], bp[3], cp[3], q[3];
  for (int k = 0; k < 3; ++k) {
    ab[k] = b[k] - a[k];
    ac[k] = c[k] - a[k];
    ap[k] = p[k] - a[k];
  }
  auto dot = [](const double* u, const double* w) { return u[0] * w[0] + u[1] * w[1] + u[2] * w[2]; };
  auto d2to = [&](const double* s) {
    const double w[3] = {p[0] - s[0], p[1] - s[1], p[2] - s[2]};
    return dot(w, w);
  };
  const double d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return dot(ap, ap);
  for (int k = 0; k < 3; ++k) bp[k] = p[k] - b[k];
  const double d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return dot(bp, bp);
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double v = d1 / (d1 - d3);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + v * ab[k];
    return d2to(q);
  }
  for (int k = 0; k < 3; ++k) cp[k] = p[k] - c[k];
  const double d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return dot(cp, cp);
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double w = d2 / (d2 - d6);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + w * ac[k];
    return d2to(q);
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && d4 - d3 >= 0.0 && d5 - d6 >= 0.0) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    for (int k = 0; k < 3; ++k) q[k] = b[k] + w * (c[k] - b[k]);
    return d2to(q);
  }
  const double den = 1.0 / (va + vb + vc);
  const double v = vb * den, w = vc * den;
  for (int k = 0; k < 3; ++k) q[k] = a[k] + ab[k] * v + ac[k] * w;
  return d2to(q);
}

// One thread per (triangle, cell of its grown box) candidate, candidates of
// triangle t at [coff[t], coff[t+1]) with x fastest: key = the cell when the
// cell's centre is within reach of the triangle (or the triangle is flat),
// else ncells (sorted after every cell); value = t.
__global__ void k_tri_candidates(const float* __restrict__ v, const TriRec* __restrict__ recs,
                                 const int* __restrict__ box, const uint32_t* __restrict__ coff, int T,
                                 uint32_t total, TriGridShape S, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    int lo = 0, hi = T - 1;  // the last triangle whose first candidate is <= i
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (coff[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    const int t = lo;
    const int* bx = box + 6 * (size_t)t;  // a0 a1 a2 b0 b1 b2
    const uint32_t local = i - coff[t];
    const uint32_t nx = (uint32_t)(bx[3] - bx[0] + 1), ny = (uint32_t)(bx[4] - bx[1] + 1);
    const int x = bx[0] + (int)(local % nx), y = bx[1] + (int)((local / nx) % ny), z = bx[2] + (int)(local / (nx * ny));
    const uint32_t cell = (uint32_t)x + (uint32_t)S.dims[0] * ((uint32_t)y + (uint32_t)S.dims[1] * (uint32_t)z);
    bool keep = true;
    const float4 pl = recs[t].plane;
    if (!(pl.x == 0.f && pl.y == 0.f && pl.z == 0.f)) {
      const float* q = v + 9 * (size_t)t;
      const double a[3] = {q[0], q[1], q[2]}, b[3] = {q[3], q[4], q[5]}, c[3] = {q[6], q[7], q[8]};
      const double cc[3] = {S.lo[0] + (x + 0.5) * S.cell, S.lo[1] + (y + 0.5) * S.cell, S.lo[2] + (z + 0.5) * S.cell};
      if (point_triangle_dist2(cc, a, b, c) > S.reach2) keep = false;  // NaN keeps the cell
    }
    keys[i] = keep ? cell : S.ncells;
    vals[i] = (uint32_t)t;
  }
}

// Entries per cell of the sorted candidates (the kept ones).
__global__ void k_tri_cell_counts(const uint32_t* __restrict__ skeys, uint32_t n, uint32_t ncells,
                                  uint32_t* __restrict__ counts) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t k = skeys[i];
    if (k < ncells) atomicAdd(&counts[k], 1u);
  }
}

int launch_triangle_grid(const float* v, const float* nrm, const uint32_t* grp, const uint32_t* mot, int T,
                         const int* box, const uint32_t* coff, uint32_t total, const TriGridShape& S,
                         TriRec* recs, uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, uint32_t* hist,
                         uint32_t* part, uint32_t* counts, uint32_t* tstart, cudaStream_t s, const uint32_t** items) {
  k_tri_records<<<grid_for((uint64_t)T, 128), 128, 0, s>>>(v, nrm, grp, mot, T, recs);
  *items = va;
  if (total == 0) {
    cudaMemsetAsync(tstart, 0, sizeof(uint32_t) * ((size_t)S.ncells + 1), s);
    return 0;
  }
  k_tri_candidates<<<grid_for(total, 256), 256, 0, s>>>(v, recs, box, coff, T, total, S, ka, va);
  int bits = 1;
  while (bits < 32 && (1ull << bits) <= (uint64_t)S.ncells) ++bits;
  const int which = launch_radix_sort(nullptr, ka, va, kb, vb, total, bits, hist, part, s);
  const uint32_t* sk = which ? kb : ka;
  *items = which ? vb : va;
  cudaMemsetAsync(counts, 0, sizeof(uint32_t) * ((size_t)S.ncells + 1), s);
  k_tri_cell_counts<<<grid_for(total, 256), 256, 0, s>>>(sk, total, S.ncells, counts);
  launch_exclusive_scan(nullptr, counts, tstart, S.ncells + 1, part, nullptr, s);
  return 0;
}

}  // namespace rp
