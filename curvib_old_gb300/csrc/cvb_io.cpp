// The files on either side of the path, read and written on the host:
//  - grid.dat, the node coordinates MG_Initial reads (init.c:339-349, 606-735);
//  - PETSc binary vectors, as VecView writes and VecLoad reads them, and the
//    restart set Ucont_P_Binary_Output / _Input (main.c:75-467) keeps in them:
//    nvfield, vfield, ufield and pfield, "<name>%05d_%1d.dat" by step and block.
// PETSc's binary vector format: the int32 class id 1211214, the int32 length,
// then the values as IEEE doubles, all big-endian.  A vector with a block size
// above one also gets "<file>.info" holding "-vecload_block_size <bs>".  On
// one rank a DMDA vector's natural order is its [k][j][i] box, so the values
// are the caller's arrays as they stand.
#include "../../include/cvb.h"

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int32_t kVecClassId = 1211214;

void put_be32(unsigned char *b, uint32_t v) {
  b[0] = (unsigned char)(v >> 24); b[1] = (unsigned char)(v >> 16);
  b[2] = (unsigned char)(v >> 8); b[3] = (unsigned char)v;
}
uint32_t get_be32(const unsigned char *b) {
  return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}
void put_be64(unsigned char *b, uint64_t v) {
  for (int q = 7; q >= 0; q--) { b[q] = (unsigned char)v; v >>= 8; }
}
uint64_t get_be64(const unsigned char *b) {
  uint64_t v = 0;
  for (int q = 0; q < 8; q++) v = (v << 8) | b[q];
  return v;
}

struct File {
  FILE *f = nullptr;
  File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
  ~File() { if (f) std::fclose(f); }
};

int vec_header(FILE *f, long long *n) {
  unsigned char h[8];
  if (std::fread(h, 1, 8, f) != 8) return CVB_BAD_INPUT;
  if ((int32_t)get_be32(h) != kVecClassId) return CVB_BAD_INPUT;
  const int32_t len = (int32_t)get_be32(h + 4);
  if (len < 0) return CVB_BAD_INPUT;
  *n = len;
  return CVB_OK;
}

std::string field_path(const char *dir, const char *name, int ti, int block) {
  char file[64];
  std::snprintf(file, sizeof file, "%s%05d_%1d.dat", name, ti, block);
  std::string p = dir && *dir ? std::string(dir) : std::string(".");
  if (p.back() != '/') p += '/';
  return p + file;
}

// One whitespace-separated number, as fscanf("%le") reads it.
bool read_number(FILE *f, double *v) {
  char tok[128];
  if (std::fscanf(f, "%127s", tok) != 1) return false;
  char *end = nullptr;
  errno = 0;
  *v = std::strtod(tok, &end);
  return end && *end == 0 && end != tok;
}

}  // namespace

extern "C" {

int cvb_petsc_vec_write(const char *path, const double *v, long long n, int block_size) {
  if (!path || (n > 0 && !v) || n < 0 || n > 0x7fffffffLL || block_size < 1) return CVB_BAD_INPUT;
  File w(path, "wb");
  if (!w.f) return CVB_BAD_INPUT;
  unsigned char h[8];
  put_be32(h, (uint32_t)kVecClassId);
  put_be32(h + 4, (uint32_t)n);
  if (std::fwrite(h, 1, 8, w.f) != 8) return CVB_BAD_INPUT;
  std::vector<unsigned char> buf(8 * 4096);
  for (long long q0 = 0; q0 < n; q0 += 4096) {
    const long long m = n - q0 < 4096 ? n - q0 : 4096;
    for (long long q = 0; q < m; q++) {
      uint64_t bits;
      std::memcpy(&bits, v + q0 + q, 8);
      put_be64(buf.data() + 8 * q, bits);
    }
    if (std::fwrite(buf.data(), 8, (size_t)m, w.f) != (size_t)m) return CVB_BAD_INPUT;
  }
  if (block_size > 1) {
    File info((std::string(path) + ".info").c_str(), "w");
    if (!info.f || std::fprintf(info.f, "-vecload_block_size %d\n", block_size) < 0) return CVB_BAD_INPUT;
  }
  return CVB_OK;
}

int cvb_petsc_vec_size(const char *path, long long *n) {
  if (!path || !n) return CVB_BAD_INPUT;
  File r(path, "rb");
  if (!r.f) return CVB_BAD_INPUT;
  return vec_header(r.f, n);
}

int cvb_petsc_vec_read(const char *path, double *v, long long n) {
  if (!path || (n > 0 && !v)) return CVB_BAD_INPUT;
  File r(path, "rb");
  if (!r.f) return CVB_BAD_INPUT;
  long long len = 0;
  if (vec_header(r.f, &len) != CVB_OK || len != n) return CVB_BAD_INPUT;
  std::vector<unsigned char> buf(8 * 4096);
  for (long long q0 = 0; q0 < n; q0 += 4096) {
    const long long m = n - q0 < 4096 ? n - q0 : 4096;
    if (std::fread(buf.data(), 8, (size_t)m, r.f) != (size_t)m) return CVB_BAD_INPUT;
    for (long long q = 0; q < m; q++) {
      const uint64_t bits = get_be64(buf.data() + 8 * q);
      std::memcpy(v + q0 + q, &bits, 8);
    }
  }
  return CVB_OK;
}

int cvb_restart_write(const char *dir, int ti, int block, long long ncells, const double *nvert, const double *ucont,
                      const double *ucat, const double *p) {
  if (ti < 0 || ti > 99999 || block < 0 || block > 9 || ncells < 1) return CVB_BAD_INPUT;
  const struct { const char *name; const double *v; int bs; } f[4] = {
      {"nvfield", nvert, 1}, {"vfield", ucont, 3}, {"ufield", ucat, 3}, {"pfield", p, 1}};
  for (const auto &e : f) {
    if (!e.v) continue;
    const int rc = cvb_petsc_vec_write(field_path(dir, e.name, ti, block).c_str(), e.v, e.bs * ncells, e.bs);
    if (rc) return rc;
  }
  return CVB_OK;
}

int cvb_restart_read(const char *dir, int ti, int block, long long ncells, double *ucont, double *p, double *nvert_o) {
  if (ti < 0 || ti > 99999 || block < 0 || block > 9 || ncells < 1) return CVB_BAD_INPUT;
  const struct { const char *name; double *v; int bs; } f[3] = {
      {"vfield", ucont, 3}, {"pfield", p, 1}, {"nvfield", nvert_o, 1}};
  for (const auto &e : f) {
    if (!e.v) continue;
    const int rc = cvb_petsc_vec_read(field_path(dir, e.name, ti, block).c_str(), e.v, e.bs * ncells);
    if (rc) return rc;
  }
  return CVB_OK;
}

int cvb_bcs_dat_read(const char *path, int nblocks, int *bctype, int *periodic) {
  if (!path || nblocks < 1 || !bctype) return CVB_BAD_INPUT;
  File r(path, "r");
  if (!r.f) return CVB_BAD_INPUT;
  int per[3] = {0, 0, 0};
  for (int b = 0; b < nblocks; b++) {
    int *t = bctype + 6 * b;
    // "%i": decimal, or 0x hexadecimal, or 0 octal, as the reference's fscanf
    if (std::fscanf(r.f, "%i %i %i %i %i %i", t, t + 1, t + 2, t + 3, t + 4, t + 5) != 6) return CVB_BAD_INPUT;
    if (t[0] == 7 || t[1] == 7) per[0] = 1;
    if (t[2] == 7 || t[3] == 7) per[1] = 1;
    if (t[4] == 7 || t[5] == 7) per[2] = 1;
  }
  if (periodic)
    for (int d = 0; d < 3; d++) periodic[d] = per[d];
  return CVB_OK;
}

int cvb_grid_dat_read(const char *path, int block, int grid1d, double cl, double l_dim, int *IM, int *JM, int *KM,
                      double *coords, long long capacity) {
  if (!path || !IM || !JM || !KM || block < 0 || !(cl != 0.0)) return CVB_BAD_INPUT;
  File r(path, "r");
  if (!r.f) return CVB_BAD_INPUT;
  int nblocks = 0;
  if (std::fscanf(r.f, "%d", &nblocks) != 1 || nblocks < 1 || block >= nblocks) return CVB_BAD_INPUT;
  std::vector<double> gc;
  for (int b = 0; b <= block; b++) {
    int im, jm, km;
    if (std::fscanf(r.f, "%d %d %d", &im, &jm, &km) != 3 || im < 2 || jm < 2 || km < 2) return CVB_BAD_INPUT;
    const long long nodes = (long long)im * jm * km;
    if (nodes > (1LL << 31)) return CVB_BAD_INPUT;
    if (b < block || !coords) {
      // skip this block's numbers (or only report the sizes)
      if (b == block) {
        *IM = im; *JM = jm; *KM = km;
        return CVB_OK;
      }
      const long long cnt = grid1d ? (long long)3 * (im + jm + km) : 3 * nodes;
      double x;
      for (long long q = 0; q < cnt; q++)
        if (!read_number(r.f, &x)) return CVB_BAD_INPUT;
      continue;
    }
    *IM = im; *JM = jm; *KM = km;
    if (capacity < 3 * nodes) return CVB_BAD_INPUT;
    if (grid1d) {
      // one "x y z" line per node of each direction, one component used each
      gc.resize((size_t)(im + jm + km));
      double x, y, z;
      for (int q = 0; q < im + jm + km; q++) {
        if (!read_number(r.f, &x) || !read_number(r.f, &y) || !read_number(r.f, &z)) return CVB_BAD_INPUT;
        gc[q] = q < im ? x : q < im + jm ? y : z;
      }
      for (int k = 0; k < km; k++)
        for (int j = 0; j < jm; j++)
          for (int i = 0; i < im; i++) {
            double *c = coords + 3 * (((size_t)k * jm + j) * im + i);
            c[0] = gc[i] / cl * l_dim;
            c[1] = gc[im + j] / cl * l_dim;
            c[2] = gc[im + jm + k] / cl * l_dim;
          }
    } else {
      // all x, then all y, then all z, each [k][j][i]
      for (int comp = 0; comp < 3; comp++)
        for (long long q = 0; q < nodes; q++) {
          double x;
          if (!read_number(r.f, &x)) return CVB_BAD_INPUT;
          coords[3 * q + comp] = x / cl * l_dim;
        }
    }
    return CVB_OK;
  }
  return CVB_BAD_INPUT;
}

}  // extern "C"
