// io.cpp -- the reference's input files on the host: grids (xyz.dat and
// grid.dat, Source/init.c:254-366), immersed-body surfaces in UCD form
// (ibmdata%02d, Source/ibm_io.c:782-1011) and PETSc binary vectors (the
// vfield / pfield / nvfield restart fields, Source/main.c:376-935, written
// by VecView and read by VecLoadIntoVector).  Plain C++ without byte-order
// intrinsics, so it builds and reads the same on x86 and Arm hosts.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vfs_poisson.h"

namespace vfs {
void set_last_error(const std::string &msg);  // poisson.cu
}

namespace {

int fail(int code, const std::string &m) {
  vfs::set_last_error(m);
  return code;
}

struct File {
  FILE *f;
  explicit File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

// PETSc writes its binary files big-endian (PetscBinaryWrite)
uint32_t load_be32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}
double load_be64(const unsigned char *p) {
  uint64_t v = 0;
  for (int q = 0; q < 8; q++) v = (v << 8) | (uint64_t)p[q];
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}
void store_be32(unsigned char *p, uint32_t v) {
  for (int q = 3; q >= 0; q--, v >>= 8) p[q] = (unsigned char)(v & 0xff);
}
void store_be64(unsigned char *p, double d) {
  uint64_t v;
  std::memcpy(&v, &d, 8);
  for (int q = 7; q >= 0; q--, v >>= 8) p[q] = (unsigned char)(v & 0xff);
}

constexpr uint32_t kVecClassId = 1211214;  // PETSc VEC_FILE_CLASSID

}  // namespace

extern "C" {

int vfs_read_petsc_vec(const char *path, int64_t *n, double *values) {
  if (!path || !n) return fail(VFS_EINVAL, "null argument");
  File f(path, "rb");
  if (!f.f) return fail(VFS_EINVAL, std::string("cannot open ") + path);
  unsigned char hdr[8];
  if (std::fread(hdr, 1, 8, f.f) != 8) return fail(VFS_EINVAL, "short PETSc vector header");
  if (load_be32(hdr) != kVecClassId) return fail(VFS_EINVAL, "not a PETSc binary vector (class id)");
  const int64_t len = (int64_t)(int32_t)load_be32(hdr + 4);
  if (len < 0) return fail(VFS_EINVAL, "negative PETSc vector length");
  if (!values) {
    *n = len;
    return VFS_OK;
  }
  if (*n < len) return fail(VFS_EINVAL, "buffer shorter than the PETSc vector");
  std::vector<unsigned char> buf(8 * 4096);
  for (int64_t done = 0; done < len;) {
    const int64_t chunk = std::min<int64_t>(4096, len - done);
    if (std::fread(buf.data(), 8, (size_t)chunk, f.f) != (size_t)chunk)
      return fail(VFS_EINVAL, "short PETSc vector data");
    for (int64_t q = 0; q < chunk; q++) values[done + q] = load_be64(&buf[8 * q]);
    done += chunk;
  }
  *n = len;
  return VFS_OK;
}

int vfs_write_petsc_vec(const char *path, int64_t n, const double *values) {
  if (!path || (!values && n > 0) || n < 0 || n > INT32_MAX) return fail(VFS_EINVAL, "bad argument");
  File f(path, "wb");
  if (!f.f) return fail(VFS_EINVAL, std::string("cannot create ") + path);
  unsigned char hdr[8];
  store_be32(hdr, kVecClassId);
  store_be32(hdr + 4, (uint32_t)n);
  if (std::fwrite(hdr, 1, 8, f.f) != 8) return fail(VFS_EINVAL, "write failed");
  std::vector<unsigned char> buf(8 * 4096);
  for (int64_t done = 0; done < n;) {
    const int64_t chunk = std::min<int64_t>(4096, n - done);
    for (int64_t q = 0; q < chunk; q++) store_be64(&buf[8 * q], values[done + q]);
    if (std::fwrite(buf.data(), 8, (size_t)chunk, f.f) != (size_t)chunk) return fail(VFS_EINVAL, "write failed");
    done += chunk;
  }
  return VFS_OK;
}

int vfs_read_grid(const char *path, int format, int block, double L_dim, double cl, int *dims, double *coor) {
  if (!path || !dims || block < 0 || !(cl != 0.)) return fail(VFS_EINVAL, "bad argument");
  if (format < 0 || format > 2) return fail(VFS_EINVAL, "format: 0 xyz.dat, 1 grid.dat text, 2 grid.dat binary");
  File f(path, format == 2 ? "rb" : "r");
  if (!f.f) return fail(VFS_EINVAL, std::string("cannot open ") + path);
  int nblock = 1;
  if (format == 1 && std::fscanf(f.f, "%i", &nblock) != 1) return fail(VFS_EINVAL, "grid.dat: block count");
  if (format == 2 && std::fread(&nblock, sizeof(int), 1, f.f) != 1) return fail(VFS_EINVAL, "grid.dat: block count");
  if (block >= nblock) return fail(VFS_EINVAL, "block index beyond the file's block count");
  for (int bi = 0; bi <= block; bi++) {
    int IM = 0, JM = 0, KM = 0;
    if (format == 2) {
      if (std::fread(&IM, sizeof(int), 1, f.f) != 1 || std::fread(&JM, sizeof(int), 1, f.f) != 1 ||
          std::fread(&KM, sizeof(int), 1, f.f) != 1)
        return fail(VFS_EINVAL, "grid.dat: dimensions");
    } else if (std::fscanf(f.f, "%i %i %i", &IM, &JM, &KM) != 3) {
      return fail(VFS_EINVAL, "grid file: dimensions");
    }
    if (IM < 2 || JM < 2 || KM < 2) return fail(VFS_EINVAL, "grid file: fewer than 2 nodes in a direction");
    const bool mine = bi == block;
    if (mine) {
      dims[0] = IM;
      dims[1] = JM;
      dims[2] = KM;
    }
    // DA layout (KM+1)(JM+1)(IM+1) x 3: node (i,j,k) at i < IM (init.c:327-360)
    const size_t mx = IM + 1, my = JM + 1;
    auto at = [&](int i, int j, int k) { return (((size_t)k * my + j) * mx + i) * 3; };
    if (format == 0) {
      std::vector<double> X(IM), Y(JM), Z(KM);
      double tmp;
      for (int i = 0; i < IM; i++)
        if (std::fscanf(f.f, "%le %le %le", &X[i], &tmp, &tmp) != 3) return fail(VFS_EINVAL, "xyz.dat: x rows");
      for (int j = 0; j < JM; j++)
        if (std::fscanf(f.f, "%le %le %le", &tmp, &Y[j], &tmp) != 3) return fail(VFS_EINVAL, "xyz.dat: y rows");
      for (int k = 0; k < KM; k++)
        if (std::fscanf(f.f, "%le %le %le", &tmp, &tmp, &Z[k]) != 3) return fail(VFS_EINVAL, "xyz.dat: z rows");
      if (mine && coor)
        for (int k = 0; k < KM; k++)
          for (int j = 0; j < JM; j++)
            for (int i = 0; i < IM; i++) {
              double *c = &coor[at(i, j, k)];
              c[0] = X[i] / cl * L_dim;
              c[1] = Y[j] / cl * L_dim;
              c[2] = Z[k] / cl * L_dim;
            }
      return VFS_OK;  // one block
    }
    for (int q = 0; q < 3; q++)
      for (int k = 0; k < KM; k++)
        for (int j = 0; j < JM; j++)
          for (int i = 0; i < IM; i++) {
            double v;
            if (format == 2 ? std::fread(&v, sizeof(double), 1, f.f) != 1 : std::fscanf(f.f, "%le", &v) != 1)
              return fail(VFS_EINVAL, "grid.dat: coordinates");
            if (mine && coor) coor[at(i, j, k) + q] = v / cl * L_dim;
          }
    if (mine) return VFS_OK;
  }
  return VFS_OK;
}

int vfs_read_ucd(const char *path, const double *place, int *n_v, int *n_elmt, double *xyz, int32_t *tri) {
  if (!path || !n_v || !n_elmt) return fail(VFS_EINVAL, "null argument");
  File f(path, "r");
  if (!f.f) return fail(VFS_EINVAL, std::string("cannot open ") + path);
  char line[512];
  for (int q = 0; q < 3; q++)
    if (!std::fgets(line, sizeof line, f.f)) return fail(VFS_EINVAL, "UCD: header lines");
  int nv = 0, ne = 0, ii;
  if (std::fscanf(f.f, "%i %i %i %i %i", &nv, &ne, &ii, &ii, &ii) != 5 || nv < 3 || ne < 1)
    return fail(VFS_EINVAL, "UCD: node and element counts");
  if (!xyz || !tri) {
    *n_v = nv;
    *n_elmt = ne;
    return VFS_OK;
  }
  if (*n_v < nv || *n_elmt < ne) return fail(VFS_EINVAL, "UCD: buffers shorter than the file's counts");
  // placement (ibm_io.c:842-890): scale L_dim, offset CM, then the initial
  // rotations about (x_r, y_r, z_r) by angle_x0, angle_y0, angle_z0 in turn
  double L = 1., cm[3] = {0., 0., 0.}, r[3] = {0., 0., 0.}, ang[3] = {0., 0., 0.};
  if (place) {
    L = place[0];
    for (int q = 0; q < 3; q++) {
      cm[q] = place[1 + q];
      r[q] = place[4 + q];
      ang[q] = place[7 + q];
    }
  }
  for (int i = 0; i < nv; i++) {
    double x, y, z;
    if (std::fscanf(f.f, "%i %le %le %le", &ii, &x, &y, &z) != 4) return fail(VFS_EINVAL, "UCD: node rows");
    x = x * L + cm[0];
    y = y * L + cm[1];
    z = z * L + cm[2];
    double x_, y_, z_;
    y_ = r[1] + (y - r[1]) * std::cos(ang[0]) - (z - r[2]) * std::sin(ang[0]);
    z_ = r[2] + (y - r[1]) * std::sin(ang[0]) + (z - r[2]) * std::cos(ang[0]);
    y = y_;
    z = z_;
    x_ = r[0] + (z - r[2]) * std::sin(ang[1]) + (x - r[0]) * std::cos(ang[1]);
    z_ = r[2] + (z - r[2]) * std::cos(ang[1]) - (x - r[0]) * std::sin(ang[1]);
    x = x_;
    z = z_;
    x_ = r[0] + (x - r[0]) * std::cos(ang[2]) - (y - r[1]) * std::sin(ang[2]);
    y_ = r[1] + (x - r[0]) * std::sin(ang[2]) + (y - r[1]) * std::cos(ang[2]);
    x = x_;
    y = y_;
    xyz[3 * i] = x;
    xyz[3 * i + 1] = y;
    xyz[3 * i + 2] = z;
  }
  for (int e = 0; e < ne; e++) {
    char kind[32];
    int a, b, c;
    if (std::fscanf(f.f, "%i %i %31s %i %i %i", &ii, &ii, kind, &a, &b, &c) != 6)
      return fail(VFS_EINVAL, "UCD: element rows");
    if (a < 1 || b < 1 || c < 1 || a > nv || b > nv || c > nv) return fail(VFS_EINVAL, "UCD: vertex index range");
    tri[3 * e] = a - 1;
    tri[3 * e + 1] = b - 1;
    tri[3 * e + 2] = c - 1;
  }
  *n_v = nv;
  *n_elmt = ne;
  return VFS_OK;
}

}  // extern "C"
