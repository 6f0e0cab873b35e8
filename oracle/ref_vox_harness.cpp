// Host harness for the reference's solid voxeliser (test infrastructure only,
// see ref_build.py).
//
// The reference's voxelize_triangle_solid kernel, its helpers and the cube
// frame of voxelize_mesh are cut out of its sources into oracle/_ref/ at build
// time and compiled here as host code.  This file supplies the CUDA keywords
// and thread coordinates, an atomicXor that is a plain xor (the emulated
// threads run one after another), and the handful of glm vector operations the
// code uses, written from glm's documented definitions:
//   dot(a, b)     = (a.x b.x + a.y b.y) + a.z b.z
//   cross(a, b)   = (a.y b.z - b.y a.z, a.z b.x - b.z a.x, a.x b.y - b.x a.y)
//   normalize(v)  = v * (1 / sqrt(dot(v, v)))
// ref_voxelize() then follows voxelize_mesh (voxelizer/voxelize_main.cpp:
// 344-406): the tight bounding box, the cube frame padded to the next power of
// two above the preferred resolution, one emulated thread per triangle, and
// the word reversal of HierarchyGrid::genFromMesh (grid/Grid.cpp:708) that
// turns the MSB-first table into LSB-first words.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#define __global__
#define __device__
#define __host__
#define __inline__ inline

struct RefDim3 { unsigned x = 0, y = 0, z = 0; };
static RefDim3 threadIdx, blockIdx, blockDim, gridDim;

static inline unsigned atomicXor(unsigned* a, unsigned v) { const unsigned o = *a; *a ^= v; return o; }
// the Morton path is never taken (morton_order = false)
static inline uint64_t mortonEncode_LUT(unsigned, unsigned, unsigned) { return 0; }

namespace glm {
struct vec2 {
  float x = 0, y = 0;
  vec2() = default;
  template <typename A, typename B> vec2(A a, B b) : x((float)a), y((float)b) {}
  float& operator[](int i) { return i ? y : x; }
  const float& operator[](int i) const { return i ? y : x; }
};
struct vec3 {
  float x = 0, y = 0, z = 0;
  vec3() = default;
  template <typename A, typename B, typename C> vec3(A a, B b, C c) : x((float)a), y((float)b), z((float)c) {}
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct uvec3 {
  unsigned x = 0, y = 0, z = 0;
  uvec3() = default;
  uvec3(unsigned a, unsigned b, unsigned c) : x(a), y(b), z(c) {}
};
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) {
  return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 normalize(vec3 v) { return v * (1.0f / std::sqrt(dot(v, v))); }
inline vec2 max(vec2 a, vec2 b) { return vec2(std::max(a.x, b.x), std::max(a.y, b.y)); }
inline vec2 min(vec2 a, vec2 b) { return vec2(std::min(a.x, b.x), std::min(a.y, b.y)); }
}  // namespace glm

#include "ref_vox_frame.inc"
#include "ref_vox.inc"

extern "C" {

// voxelize_mesh with the GPU routine's arithmetic: verts[3 nverts], tris[3 ntris];
// writes the resolution, the cube frame (min xyz, max xyz) and reso^3 / 32
// LSB-first words (words must hold them; reso is at most 2 * prefer).
int ref_voxelize(const float* verts, int nverts, const int* tris, int ntris, int prefer, int* reso_out,
                 float* box_out, unsigned* words, size_t cap) {
  std::vector<float> vc(verts, verts + 3 * (size_t)nverts);
  std::vector<int> ids(tris, tris + 3 * (size_t)ntris);
  auto vbb = get_point_bb(vc);
  std::pair<glm::vec3, glm::vec3> out_bb;
  const int reso = padd2SatifyResolution(prefer, vbb, out_bb);
  AABox<glm::vec3> bcube(out_bb.first, out_bb.second);
  voxinfo info(bcube, glm::uvec3(reso, reso, reso), ids.size() / 3);
  const size_t nwords = (size_t)reso * reso * reso / 32;
  if (nwords > cap) return -1;
  std::vector<float> tri;
  for (size_t i = 0; i < ids.size(); i += 3)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) tri.push_back(vc[(size_t)ids[i + k] * 3 + c]);
  std::vector<unsigned> table(nwords, 0u);
  // one thread per triangle (the reference's launch: blocks of 256)
  blockDim.x = 256;
  gridDim.x = (unsigned)((ntris + 255) / 256);
  for (int t = 0; t < ntris; ++t) {
    blockIdx.x = t / 256;
    threadIdx.x = t % 256;
    // a thread of the reference launch whose index is below n_triangles runs
    // its one triangle (stride = the grid, at least n_triangles)
    voxelize_triangle_solid(info, tri.data(), table.data(), false);
  }
  for (size_t w = 0; w < nwords; ++w) {
    unsigned v = table[w], r = 0;
    for (int b = 0; b < 32; ++b) r |= ((v >> b) & 1u) << (31 - b);
    words[w] = r;
  }
  *reso_out = reso;
  for (int i = 0; i < 3; ++i) {
    box_out[i] = bcube.min[i];
    box_out[3 + i] = bcube.max[i];
  }
  return 0;
}

}  // extern "C"
