// Files and the reference's domain input: bit-mask domains, raw array
// records, active-element records, and checkpoints that resume a design run
// bit for bit.
//
// The reference reads its domain as an LSB-first uint32 bit mask over a
// power-of-two cube (HierarchyGrid::genFromMesh, grid/Grid.cpp:977), writes
// arrays as raw binary records (bio::write_vector, utils/binaryIO.h:70-108;
// HierarchyGrid::writeCoeff, grid/Grid.cpp:2139-2156, in FP32) and writes the
// density of the active elements with their cell positions
// (HierarchyGrid::writeDensity, grid/Grid.cpp:1266-1310, handed to OpenVDB,
// which is not part of this library: the same (x, y, z, value) records are
// written as a raw record instead).  It has no checkpoint; a run restarts
// from a coefficient file.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "handle.h"

using namespace topo;

namespace {

int io_fail(topo_handle* h, int code, const std::string& msg) { return handle_fail(h, code, msg.c_str()); }

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) : f(path ? std::fopen(path, mode) : nullptr) {}
  ~File() { if (f) std::fclose(f); }
  bool put(const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
  bool get(void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }
};

bool bit_at(const uint32_t* words, int64_t b) { return (words[b >> 5] >> (b & 31)) & 1u; }

// device array -> host vector (blocking, on the handle's stream)
template <typename T>
bool download(cudaStream_t s, const T* d, size_t n, std::vector<T>& out) {
  out.resize(n);
  if (n == 0) return true;
  return cudaMemcpyAsync(out.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaStreamSynchronize(s) == cudaSuccess;
}
template <typename T>
bool upload(cudaStream_t s, T* d, const std::vector<T>& in) {
  if (in.empty()) return true;
  return cudaMemcpyAsync(d, in.data(), sizeof(T) * in.size(), cudaMemcpyHostToDevice, s) == cudaSuccess &&
         cudaStreamSynchronize(s) == cudaSuccess;
}

constexpr char kMagic[8] = {'T', 'O', 'P', 'O', 'C', 'K', 'P', '1'};

}  // namespace

extern "C" {

int topo_bitmask_to_eactive(const int* reso3, const uint32_t* words, int nx, int ny, int nz, uint8_t* eactive) {
  if (!reso3 || !words || !eactive || nx < 1 || ny < 1 || nz < 1) return TOPO_E_BAD_INPUT;
  const int64_t rx = reso3[0], ry = reso3[1], rz = reso3[2];
  if (rx < nx || ry < ny || rz < nz) return TOPO_E_BAD_INPUT;
  const int64_t nbits = rx * ry * rz;
  // every set bit must lie inside the nx x ny x nz box at the frame's origin
  for (int64_t w = 0; w < (nbits + 31) / 32; ++w) {
    uint32_t word = words[w];
    if (w == (nbits - 1) / 32 && (nbits & 31)) word &= (1u << (nbits & 31)) - 1u;
    while (word) {
      const int b = __builtin_ctz(word);
      word &= word - 1;
      const int64_t id = 32 * w + b;
      const int64_t x = id % rx, y = (id / rx) % ry, z = id / (rx * ry);
      if (x >= nx || y >= ny || z >= nz) return TOPO_E_BAD_INPUT;
    }
  }
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x)
        eactive[x + nx * (y + ny * z)] = bit_at(words, x + rx * (y + ry * z)) ? 1 : 0;
  return TOPO_OK;
}

int topo_eactive_to_bitmask(int nx, int ny, int nz, const uint8_t* eactive, const int* reso3, uint32_t* words) {
  if (!reso3 || !words || nx < 1 || ny < 1 || nz < 1) return TOPO_E_BAD_INPUT;
  const int64_t rx = reso3[0], ry = reso3[1], rz = reso3[2];
  if (rx < nx || ry < ny || rz < nz) return TOPO_E_BAD_INPUT;
  std::memset(words, 0, sizeof(uint32_t) * (size_t)((rx * ry * rz + 31) / 32));
  for (int64_t z = 0; z < nz; ++z)
    for (int64_t y = 0; y < ny; ++y)
      for (int64_t x = 0; x < nx; ++x)
        if (!eactive || eactive[x + nx * (y + ny * z)]) {
          const int64_t b = x + rx * (y + ry * z);
          words[b >> 5] |= 1u << (b & 31);
        }
  return TOPO_OK;
}

int topo_create_bitmask(const topo_config* cfg, const int* reso3, const uint32_t* words, topo_handle** out) {
  if (!cfg || !out) return TOPO_E_BAD_INPUT;
  std::vector<uint8_t> ea((size_t)cfg->nx * cfg->ny * cfg->nz);
  const int rc = topo_bitmask_to_eactive(reso3, words, cfg->nx, cfg->ny, cfg->nz, ea.data());
  if (rc != TOPO_OK) return rc;
  return topo_create(cfg, ea.data(), out);
}

int topo_write_array(topo_handle* h, int which, int level, const char* path, int fp32) {
  if (!h || !path) return TOPO_E_BAD_INPUT;
  size_t n = 0;
  void* dp = nullptr;
  int rc = topo_array_size(h, which, level, &n);
  if (rc == TOPO_OK) rc = topo_device_ptr(h, which, level, &dp);
  if (rc != TOPO_OK) return rc;
  if (which == TOPO_VMASK || which == TOPO_EACTIVE) {
    std::vector<uint8_t> b(n);
    RET_IF(topo_get_array(h, which, level, b.data(), n));
    File f(path, "wb");
    if (!f.f || !f.put(b.data(), n)) return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot write ") + path);
    return TOPO_OK;
  }
  std::vector<double> v(n);
  RET_IF(topo_get_array(h, which, level, v.data(), n));
  File f(path, "wb");
  if (!f.f) return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot open ") + path);
  if (fp32) {
    std::vector<float> s(v.begin(), v.end());
    if (!f.put(s.data(), sizeof(float) * n)) return io_fail(h, TOPO_E_BAD_INPUT, "short write");
  } else if (!f.put(v.data(), sizeof(double) * n)) {
    return io_fail(h, TOPO_E_BAD_INPUT, "short write");
  }
  return TOPO_OK;
}

int topo_read_array(topo_handle* h, int which, int level, const char* path, int fp32) {
  if (!h || !path || which == TOPO_VMASK || which == TOPO_EACTIVE) return TOPO_E_BAD_INPUT;
  size_t n = 0;
  RET_IF(topo_array_size(h, which, level, &n));
  File f(path, "rb");
  if (!f.f) return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot open ") + path);
  std::fseek(f.f, 0, SEEK_END);
  const long len = std::ftell(f.f);
  std::fseek(f.f, 0, SEEK_SET);
  const size_t es = fp32 ? sizeof(float) : sizeof(double);
  if (len < 0 || (size_t)len != n * es)
    return io_fail(h, TOPO_E_BAD_INPUT, std::string("record size does not match the array: ") + path);
  std::vector<double> v(n);
  if (fp32) {
    std::vector<float> s(n);
    if (!f.get(s.data(), sizeof(float) * n)) return io_fail(h, TOPO_E_BAD_INPUT, "short read");
    for (size_t i = 0; i < n; ++i) v[i] = s[i];
  } else if (!f.get(v.data(), sizeof(double) * n)) {
    return io_fail(h, TOPO_E_BAD_INPUT, "short read");
  }
  return topo_put_array(h, which, level, v.data(), n);
}

int topo_write_active_records(topo_handle* h, int which, const char* path, int64_t* count) {
  if (!h || !path || (which != TOPO_RHO && which != TOPO_SENS)) return TOPO_E_BAD_INPUT;
  int dims[3];
  RET_IF(topo_level_dims(h, 0, dims, nullptr));
  const int64_t ne = (int64_t)dims[0] * dims[1] * dims[2];
  std::vector<double> v(ne);
  std::vector<uint8_t> ea(ne);
  RET_IF(topo_get_array(h, which, 0, v.data(), ne));
  RET_IF(topo_get_array(h, TOPO_EACTIVE, 0, ea.data(), ne));
  std::vector<float> rec;
  rec.reserve(4 * (size_t)ne);
  int64_t k = 0;
  for (int64_t z = 0; z < dims[2]; ++z)
    for (int64_t y = 0; y < dims[1]; ++y)
      for (int64_t x = 0; x < dims[0]; ++x) {
        const int64_t e = x + dims[0] * (y + dims[1] * z);
        if (!ea[e]) continue;
        rec.push_back((float)x); rec.push_back((float)y); rec.push_back((float)z); rec.push_back((float)v[e]);
        ++k;
      }
  File f(path, "wb");
  if (!f.f || !f.put(rec.data(), sizeof(float) * rec.size()))
    return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot write ") + path);
  if (count) *count = k;
  return TOPO_OK;
}

int topo_checkpoint_save(topo_handle* h, const char* path, const void* user, size_t user_bytes) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !path || (user_bytes && !user)) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return io_fail(h, TOPO_E_STATE, "checkpoint: spline not set");
  const cudaStream_t s = h->stream;
  const LevelDims& d0 = h->lv[0].d;
  const int nl = (int)h->lv.size();
  const int64_t nc = (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
  File f(path, "wb");
  if (!f.f) return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot open ") + path);
  const int32_t hdr[8] = {1, d0.ex, d0.ey, d0.ez, nl, (int32_t)nc, h->sd.order, h->fine_df};
  // the FP32 depth carries the tensor-core and tile-height choices as flags
  const int32_t tiles[2] = {h->tz32 | (h->fine_tc ? TOPO_FINE_TC_FLAG : 0) | fine_rows_flag(h->rows32), h->tz64};
  std::vector<double> coeff, rho, u;
  if (!download(s, h->coeff, nc, coeff) || !download(s, h->rho, d0.ne, rho) ||
      !download(s, h->lv[0].U, 3 * d0.nv, u))
    return io_fail(h, TOPO_E_CUDA, "checkpoint: download");
  bool ok = f.put(kMagic, 8) && f.put(hdr, sizeof(hdr)) && f.put(tiles, sizeof(tiles)) &&
            f.put(coeff.data(), sizeof(double) * nc) && f.put(rho.data(), sizeof(double) * d0.ne) &&
            f.put(u.data(), sizeof(double) * 3 * d0.nv);
  for (int l = 0; ok && l < nl; ++l) {
    const DevLevel& L = h->lv[l];
    const int64_t n3 = 3 * L.d.nv;
    const double lp[2] = {L.lprev, L.lprev32};
    const uint8_t has[2] = {(uint8_t)(L.eig != nullptr), (uint8_t)(L.eig32 != nullptr)};
    ok = f.put(lp, sizeof(lp)) && f.put(has, sizeof(has));
    if (ok && L.eig) {
      std::vector<double> e;
      ok = download(s, L.eig, n3, e) && f.put(e.data(), sizeof(double) * n3);
    }
    if (ok && L.eig32) {
      std::vector<float> e;
      ok = download(s, L.eig32, n3, e) && f.put(e.data(), sizeof(float) * n3);
    }
  }
  const uint64_t ub = user_bytes;
  ok = ok && f.put(&ub, sizeof(ub)) && f.put(user, user_bytes);
  if (!ok) return io_fail(h, TOPO_E_BAD_INPUT, std::string("checkpoint: write failed: ") + path);
  return TOPO_OK;
}

int topo_checkpoint_load(topo_handle* h, const char* path, void* user, size_t user_cap, size_t* user_bytes) {
  DeviceScope scope(h ? h->cfg.device : -1);
  if (!h || !path) return TOPO_E_BAD_INPUT;
  if (!h->spline_set) return io_fail(h, TOPO_E_STATE, "checkpoint: set the spline before loading");
  const cudaStream_t s = h->stream;
  const LevelDims& d0 = h->lv[0].d;
  const int nl = (int)h->lv.size();
  const int64_t nc = (int64_t)h->sd.nb[0] * h->sd.nb[1] * h->sd.nb[2];
  File f(path, "rb");
  if (!f.f) return io_fail(h, TOPO_E_BAD_INPUT, std::string("cannot open ") + path);
  char magic[8];
  int32_t hdr[8], tiles[2];
  if (!f.get(magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !f.get(hdr, sizeof(hdr)) || !f.get(tiles, sizeof(tiles)))
    return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: not a checkpoint file");
  if (hdr[0] != 1 || hdr[1] != d0.ex || hdr[2] != d0.ey || hdr[3] != d0.ez || hdr[4] != nl || hdr[5] != nc ||
      hdr[6] != h->sd.order)
    return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: grid, levels or spline differ from the handle's");
  std::vector<double> coeff(nc), rho(d0.ne), u(3 * d0.nv);
  if (!f.get(coeff.data(), sizeof(double) * nc) || !f.get(rho.data(), sizeof(double) * d0.ne) ||
      !f.get(u.data(), sizeof(double) * 3 * d0.nv))
    return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated");
  struct LevelState { double lp[2]; uint8_t has[2]; std::vector<double> e; std::vector<float> e32; };
  std::vector<LevelState> ls(nl);
  for (int l = 0; l < nl; ++l) {
    const int64_t n3 = 3 * h->lv[l].d.nv;
    if (!f.get(ls[l].lp, sizeof(ls[l].lp)) || !f.get(ls[l].has, sizeof(ls[l].has)))
      return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated");
    if (ls[l].has[0]) { ls[l].e.resize(n3); if (!f.get(ls[l].e.data(), sizeof(double) * n3)) return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated"); }
    if (ls[l].has[1]) { ls[l].e32.resize(n3); if (!f.get(ls[l].e32.data(), sizeof(float) * n3)) return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated"); }
  }
  uint64_t ub = 0;
  if (!f.get(&ub, sizeof(ub))) return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated");
  if (user_bytes) *user_bytes = ub;
  if (ub) {
    std::vector<char> blob(ub);
    if (!f.get(blob.data(), ub)) return io_fail(h, TOPO_E_BAD_INPUT, "checkpoint: truncated");
    if (user) std::memcpy(user, blob.data(), std::min<size_t>(ub, user_cap));
  }
  // state: coefficients, density, warm start, spectral-bound warm starts, tiles
  RET_IF(topo_put_array(h, TOPO_COEFF, 0, coeff.data(), nc));
  RET_IF(topo_put_array(h, TOPO_RHO, 0, rho.data(), d0.ne));
  RET_IF(topo_put_array(h, TOPO_U, 0, u.data(), 3 * d0.nv));
  for (int l = 0; l < nl; ++l) {
    DevLevel& L = h->lv[l];
    const int64_t n3 = 3 * L.d.nv;
    L.lprev = ls[l].lp[0];
    L.lprev32 = ls[l].lp[1];
    L.lmax = 0;
    L.lmax32 = 0;
    for (int p = 0; p < 2; ++p) {
      void** slot = p == 0 ? (void**)&L.eig : (void**)&L.eig32;
      const size_t es = p == 0 ? sizeof(double) : sizeof(float);
      if (!ls[l].has[p]) continue;
      if (!*slot) {
        if (cudaMalloc(slot, es * n3) != cudaSuccess) { cudaGetLastError(); *slot = nullptr; return io_fail(h, TOPO_E_NOMEM, "checkpoint: eig"); }
        h->allocs.push_back(*slot);
      }
      const void* src = p == 0 ? (const void*)ls[l].e.data() : (const void*)ls[l].e32.data();
      if (cudaMemcpyAsync(*slot, src, es * n3, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return io_fail(h, TOPO_E_CUDA, "checkpoint: upload");
    }
  }
  // the previous estimates also in the device slots the restart test reads
  std::vector<double> lp(2 * S_MAXLEV, 0.0);
  for (int l = 0; l < nl && l < S_MAXLEV; ++l) {
    lp[l] = h->lv[l].lprev;
    lp[S_MAXLEV + l] = h->lv[l].lprev32;
  }
  if (cudaMemcpyAsync(h->sc + S_LPREV, lp.data(), sizeof(double) * lp.size(), cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return io_fail(h, TOPO_E_CUDA, "checkpoint: upload");
  if (cudaStreamSynchronize(s) != cudaSuccess) return io_fail(h, TOPO_E_CUDA, "checkpoint: upload");
  h->tz32 = tiles[0] & ~TOPO_FINE_FLAGS;
  h->fine_tc = (tiles[0] & TOPO_FINE_TC_FLAG) != 0;
  h->rows32 = (tiles[0] & TOPO_FINE_ROWS4_FLAG) ? 4 : (tiles[0] & TOPO_FINE_ROWS16_FLAG) ? 16 : 8;
  h->tz64 = tiles[1];
  h->rhop_stale = true;
  h->ops_ready = false;
  h->coarse_valid = false;
  return TOPO_OK;
}

}  // extern "C"
