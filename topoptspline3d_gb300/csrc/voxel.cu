// Solid voxelisation of a closed triangle mesh into the reference's domain bit
// mask (the mesh -> bit-mask step of voxelizer/voxelize_main.cpp:344-406).
//
// The rule is the reference's (voxelizer/voxelize_solid.cu:78-166, after
// Schwarz and Seidel): the frame is a cube around the mesh's bounding box,
// padded to the next power of two above the preferred resolution; for every
// triangle that is not parallel to x, every voxel column (y, z) whose centre
// falls inside the triangle's yz projection (edges by the top-left rule) has
// the parity of the voxels x = 0 .. xmax flipped, xmax the voxel below the
// triangle's x at that centre.  A voxel is solid when an odd number of
// triangles lie beyond it along x.
//
// The reference flips xmax + 1 bits per covered column with atomics.  Here a
// triangle toggles one marker bit, at xmax, and a second kernel turns the
// markers into the solid mask by a suffix parity along x (a voxel is solid
// when the markers at and above it have odd parity): one atomic per covered
// column instead of up to `resolution`, and 32 voxels per word in the scan.
// The arithmetic of each test is the reference's, operation for operation in
// FP32 without fused multiply-adds (this file is compiled with -fmad=false),
// so the masks are the same bits.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "topo_internal.h"

using namespace topo;

namespace {

struct V2 { float x, y; };
struct V3 { float x, y, z; };

__device__ __forceinline__ V2 sub2(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

// 1, 2, 3: the point lies on edge (v0 v1), (v1 v2), (v2 v0); 0 inside; -1 outside
__device__ int point_in_triangle(V2 v0, V2 v1, V2 v2, V2 p) {
  const V2 pa = sub2(p, v0), pb = sub2(p, v1), pc = sub2(p, v2);
  const float t1 = pa.x * pb.y - pa.y * pb.x;
  if (fabsf(t1) < 0.000001 && pa.x * pb.x <= 0 && pa.y * pb.y <= 0) return 1;
  const float t2 = pb.x * pc.y - pb.y * pc.x;
  if (fabsf(t2) < 0.000001 && pb.x * pc.x <= 0 && pb.y * pc.y <= 0) return 2;
  const float t3 = pc.x * pa.y - pc.y * pa.x;
  if (fabsf(t3) < 0.000001 && pc.x * pa.x <= 0 && pc.y * pa.y <= 0) return 3;
  return (t1 * t2 > 0 && t1 * t3 > 0) ? 0 : -1;
}

// an edge (a -> b) of a counter-clockwise triangle that owns the points on it
__device__ __forceinline__ bool top_left(V2 a, V2 b) { return (b.y < a.y) || (b.y == a.y && a.x > b.x); }

__global__ void k_vox_markers(int ntri, const float* __restrict__ tri, V3 bmin, V3 unit, int reso,
                              unsigned* __restrict__ marks) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntri) return;
  const float* q = tri + 9 * (size_t)t;
  const V3 v0 = sub3({q[0], q[1], q[2]}, bmin);
  const V3 v1 = sub3({q[3], q[4], q[5]}, bmin);
  const V3 v2 = sub3({q[6], q[7], q[8]}, bmin);
  const V3 e0 = sub3(v1, v0), e1 = sub3(v2, v1);
  // unit normal (cross product, then times 1 / sqrt of its squared length)
  const V3 c = {e0.y * e1.z - e1.y * e0.z, e0.z * e1.x - e1.z * e0.x, e0.x * e1.y - e1.x * e0.y};
  const float inv = 1.0f / sqrtf((c.x * c.x + c.y * c.y) + c.z * c.z);
  const V3 n = {c.x * inv, c.y * inv, c.z * inv};
  if (fabsf(n.x) < 0.000001) return;  // parallel to the x rays
  V2 a = {v0.y, v0.z}, b = {v1.y, v1.z}, d = {v2.y, v2.z};
  {  // counter-clockwise in the yz plane
    const V2 f0 = sub2(b, a), f1 = sub2(d, a);
    if (!(f0.x * f1.y - f1.x * f0.y > 0)) { const V2 s = b; b = d; d = s; }
  }
  const V2 hi = {fmaxf(a.x, fmaxf(b.x, d.x)), fmaxf(a.y, fmaxf(b.y, d.y))};
  const V2 lo = {fminf(a.x, fminf(b.x, d.x)), fminf(a.y, fminf(b.y, d.y))};
  const int y1 = (int)(float)floor((double)(hi.x / unit.y) - 0.5);
  const int z1 = (int)(float)floor((double)(hi.y / unit.z) - 0.5);
  const int y0 = (int)(float)ceil((double)(lo.x / unit.y) - 0.5);
  const int z0 = (int)(float)ceil((double)(lo.y / unit.z) - 0.5);
  for (int y = max(y0, 0); y <= min(y1, reso - 1); ++y)
    for (int z = max(z0, 0); z <= min(z1, reso - 1); ++z) {
      const V2 p = {(float)((y + 0.5) * (double)unit.y), (float)((z + 0.5) * (double)unit.z)};
      const int k = point_in_triangle(a, b, d, p);
      if (!((k == 1 && top_left(a, b)) || (k == 2 && top_left(b, d)) || (k == 3 && top_left(d, a)) || k == 0))
        continue;
      const float xc = (-(n.y * (p.x - v0.y) + n.z * (p.y - v0.z)) / n.x + v0.x);
      int xmax = (int)((double)(xc / unit.x) - 0.5);
      if (xmax < 0) continue;  // the reference's loop over x = 0 .. xmax runs no step
      xmax = min(xmax, reso - 1);
      const size_t loc = (size_t)xmax + (size_t)reso * ((size_t)y + (size_t)reso * z);
      atomicXor(&marks[loc >> 5], 1u << (loc & 31));
    }
}

// One thread per column (y, z) of a frame whose columns span whole words:
// solid bit x = parity of the markers at x .. reso-1.
__global__ void k_vox_scan_words(int reso, const unsigned* __restrict__ marks, unsigned* __restrict__ out) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (int64_t)reso * reso) return;
  const int wpc = reso >> 5;
  const unsigned* m = marks + col * wpc;
  unsigned* o = out + col * wpc;
  unsigned carry = 0;  // parity of the markers above the current word
  for (int w = wpc - 1; w >= 0; --w) {
    unsigned s = m[w];
    s ^= s >> 1; s ^= s >> 2; s ^= s >> 4; s ^= s >> 8; s ^= s >> 16;  // bit i: parity of bits i..31
    if (carry) s = ~s;
    o[w] = s;
    carry = s & 1u;
  }
}

// Frames under 32 voxels a side: columns share words, one bit at a time.
__global__ void k_vox_scan_bits(int reso, const unsigned* __restrict__ marks, unsigned* __restrict__ out) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= (int64_t)reso * reso) return;
  unsigned par = 0;
  for (int x = reso - 1; x >= 0; --x) {
    const size_t loc = (size_t)x + (size_t)reso * col;
    par ^= (marks[loc >> 5] >> (loc & 31)) & 1u;
    if (par) atomicOr(&out[loc >> 5], 1u << (loc & 31));
  }
}

}  // namespace

extern "C" {

int topo_voxel_frame(const float* verts, int nverts, int preferred_resolution, int* reso_out, float* box6_out) {
  if (!verts || nverts < 1 || preferred_resolution < 1 || !reso_out || !box6_out) return TOPO_E_BAD_INPUT;
  // tight bounding box (voxelizer/voxelize_main.cpp:292-310)
  float mn[3], mx[3];
  for (int j = 0; j < 3; ++j) { mn[j] = std::numeric_limits<float>::infinity(); mx[j] = -mn[j]; }
  for (int i = 0; i < nverts; ++i)
    for (int j = 0; j < 3; ++j) {
      mn[j] = std::min(mn[j], verts[3 * i + j]);
      mx[j] = std::max(mx[j], verts[3 * i + j]);
    }
  // the cube frame: next power of two above the preferred resolution, the
  // longest side scaled by reso / preferred, centred (voxelize_main.cpp:312-341)
  unsigned reso = 1;
  for (int i = 0; i < 32 && !(preferred_resolution < (int)reso); ++i) reso <<= 1;
  if (reso > 2048) return TOPO_E_BAD_INPUT;
  float len[3];
  for (int j = 0; j < 3; ++j) len[j] = mx[j] - mn[j];
  const float max_len = std::max(std::max(len[0], len[1]), len[2]);
  if (!(max_len > 0)) return TOPO_E_BAD_INPUT;
  for (int j = 0; j < 3; ++j) {
    const float pad = max_len * (int)reso / preferred_resolution;
    box6_out[j] = mn[j] - (pad - len[j]) / 2;
    box6_out[3 + j] = mx[j] + (pad - len[j]) / 2;
  }
  *reso_out = (int)reso;
  return TOPO_OK;
}

int topo_voxelize_mesh(int device, const float* verts, int nverts, const int* tris, int ntris, int preferred_resolution,
                       int* reso_out, float* box6_out, uint32_t* words, size_t nwords_cap) {
  if (!tris || ntris < 1) return TOPO_E_BAD_INPUT;
  int reso = 0;
  float box[6];
  int rc = topo_voxel_frame(verts, nverts, preferred_resolution, &reso, box);
  if (rc != TOPO_OK) return rc;
  *reso_out = reso;
  std::copy(box, box + 6, box6_out);
  const size_t nwords = (size_t)reso * reso * reso / 32 + ((size_t)reso * reso * reso % 32 ? 1 : 0);
  if (!words) return TOPO_OK;  // size query
  if (nwords_cap < nwords) return TOPO_E_BAD_INPUT;
  std::vector<float> tri(9 * (size_t)ntris);
  for (int t = 0; t < ntris; ++t)
    for (int k = 0; k < 3; ++k) {
      const int v = tris[3 * t + k];
      if (v < 0 || v >= nverts) return TOPO_E_BAD_INPUT;
      for (int c = 0; c < 3; ++c) tri[9 * (size_t)t + 3 * k + c] = verts[3 * (size_t)v + c];
    }
  DeviceScope scope(device);
  cudaStream_t s = nullptr;
  float* dtri = nullptr;
  unsigned *marks = nullptr, *out = nullptr;
  struct Free {
    cudaStream_t* s; float** t; unsigned** m; unsigned** o;
    ~Free() { if (*t) cudaFree(*t); if (*m) cudaFree(*m); if (*o) cudaFree(*o); if (*s) cudaStreamDestroy(*s); }
  } guard{&s, &dtri, &marks, &out};
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&dtri, sizeof(float) * tri.size()) != cudaSuccess ||
      cudaMalloc(&marks, sizeof(unsigned) * nwords) != cudaSuccess ||
      cudaMalloc(&out, sizeof(unsigned) * nwords) != cudaSuccess) {
    cudaGetLastError();
    return TOPO_E_NOMEM;
  }
  const V3 bmin = {box[0], box[1], box[2]};
  const V3 unit = {(box[3] - box[0]) / float(reso), (box[4] - box[1]) / float(reso), (box[5] - box[2]) / float(reso)};
  cudaMemcpyAsync(dtri, tri.data(), sizeof(float) * tri.size(), cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(marks, 0, sizeof(unsigned) * nwords, s);
  cudaMemsetAsync(out, 0, sizeof(unsigned) * nwords, s);
  k_vox_markers<<<(ntris + 127) / 128, 128, 0, s>>>(ntris, dtri, bmin, unit, reso, marks);
  const int64_t cols = (int64_t)reso * reso;
  if (reso % 32 == 0) k_vox_scan_words<<<(unsigned)((cols + 255) / 256), 256, 0, s>>>(reso, marks, out);
  else k_vox_scan_bits<<<(unsigned)((cols + 255) / 256), 256, 0, s>>>(reso, marks, out);
  count_launch(2);
  cudaMemcpyAsync(words, out, sizeof(unsigned) * nwords, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) return TOPO_E_CUDA;
  return TOPO_OK;
}

}  // extern "C"
