// tpls_backup.cu -- the reference's text backup and restart files
// (io.F90:647-716 backup_channel, io.F90:721-791 dataload_channel), written
// from and read into a context's device state, plus host-array versions
// with the reference routines' argument lists.  Host code only.
//
// Layout (l = nx+1, m = ny+1, n = nz+1, Fortran loop order, i fastest), one
// record per point:
//   k = 0..n-2:  u2, conv0_u, conv1_u
//   k = 0..n-2:  v2, conv0_v, conv1_v
//   k = 0..n-1:  w2, conv0_w, conv1_w
//   k = 0..n:    phi, conv0_phi, conv1_phi
//   k = 0..n:    pres, pres_old
// Values are written with 17 significant digits (exact for doubles), so a
// save / load round trip restores the state bit for bit.  The reference's
// backup leaves out the AB3 history of the surface-tension force (csf0,
// csf1), which a restart needs to continue the same run; it goes to a
// companion file of the same style (csf_u0, csf_u1 / csf_v0, csf_v1 /
// csf_w0, csf_w1 records over the u, v and w grids).  The reader takes any
// list-directed form of the numbers: whitespace or comma separated,
// E or D exponents, and r*value repeat counts.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tpls_gpu.h"

namespace {

struct Block {
  int nplanes;          // z planes of the block's grid
  const double *a[3];   // arrays of the record (2 or 3)
  double *w[3];         // the same for reading
  int narr;
};

// one value as " %24.16E": sign, 17 significant digits, exponent with at
// least two digits
void put_num(std::string &out, double v) {
  char buf[40];
  const int n = std::snprintf(buf, sizeof buf, " %24.16E", v);
  out.append(buf, (size_t)n);
}

int write_blocks(const char *filename, int nx, int ny, const std::vector<Block> &blocks) {
  if (!filename) return TPLS_ERR_ARG;
  FILE *f = std::fopen(filename, "wb");
  if (!f) return TPLS_ERR_IO;
  const size_t row = (size_t)(nx + 2), plane = row * (size_t)(ny + 2);
  std::string out;
  out.reserve(1 << 22);
  int rc = TPLS_OK;
  for (const Block &b : blocks) {
    const size_t npts = plane * (size_t)b.nplanes;
    for (size_t c = 0; c < npts && rc == TPLS_OK; c++) {
      for (int q = 0; q < b.narr; q++) put_num(out, b.a[q][c]);
      out.push_back('\n');
      if (out.size() > (1u << 22)) {
        if (std::fwrite(out.data(), 1, out.size(), f) != out.size()) rc = TPLS_ERR_IO;
        out.clear();
      }
    }
  }
  if (rc == TPLS_OK && !out.empty() && std::fwrite(out.data(), 1, out.size(), f) != out.size()) rc = TPLS_ERR_IO;
  if (std::fclose(f) != 0 && rc == TPLS_OK) rc = TPLS_ERR_IO;
  return rc;
}

// Sequential list-directed number reader over a whole file.
struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  double rep_val = 0.0;
  long rep_left = 0;

  bool open(const char *filename) {
    FILE *f = std::fopen(filename, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
      std::fclose(f);
      return false;
    }
    buf.resize((size_t)n + 1);
    const size_t got = std::fread(buf.data(), 1, (size_t)n, f);
    std::fclose(f);
    buf[got] = '\0';
    buf.resize(got + 1);
    for (char &ch : buf)
      if (ch == 'D' || ch == 'd') ch = 'E';  // Fortran double-precision exponents
    return true;
  }
  bool next(double *v) {
    if (rep_left > 0) {
      rep_left--;
      *v = rep_val;
      return true;
    }
    const char *s = buf.data();
    while (s[pos] == ' ' || s[pos] == '\t' || s[pos] == '\n' || s[pos] == '\r' || s[pos] == ',') pos++;
    if (s[pos] == '\0') return false;
    char *end = nullptr;
    // r*value repeat count
    const char *star = nullptr;
    for (size_t p = pos; s[p] >= '0' && s[p] <= '9'; p++)
      if (s[p + 1] == '*') star = s + p + 1;
    if (star) {
      const long r = std::strtol(s + pos, nullptr, 10);
      errno = 0;
      const double val = std::strtod(star + 1, &end);
      if (end == star + 1 || r < 1) return false;
      pos = (size_t)(end - s);
      rep_val = val;
      rep_left = r - 1;
      *v = val;
      return true;
    }
    const double val = std::strtod(s + pos, &end);
    if (end == s + pos) return false;
    pos = (size_t)(end - s);
    *v = val;
    return true;
  }
};

int read_blocks(const char *filename, int nx, int ny, const std::vector<Block> &blocks) {
  if (!filename) return TPLS_ERR_ARG;
  Reader r;
  if (!r.open(filename)) return TPLS_ERR_IO;
  const size_t plane = (size_t)(nx + 2) * (size_t)(ny + 2);
  for (const Block &b : blocks) {
    const size_t npts = plane * (size_t)b.nplanes;
    for (size_t c = 0; c < npts; c++)
      for (int q = 0; q < b.narr; q++)
        if (!r.next(&b.w[q][c])) return TPLS_ERR_IO;
  }
  return TPLS_OK;
}

bool dims_ok(const int *l, const int *m, const int *n) {
  return l && m && n && *l >= 2 && *m >= 2 && *n >= 3;
}

std::vector<Block> main_blocks(int nz, const double *u2, const double *v2, const double *w2, const double *c0u,
                               const double *c1u, const double *c0v, const double *c1v, const double *c0w,
                               const double *c1w, const double *pres_old, const double *pres, const double *phi,
                               const double *c0p, const double *c1p) {
  std::vector<Block> b(5);
  b[0] = {nz, {u2, c0u, c1u}, {const_cast<double *>(u2), const_cast<double *>(c0u), const_cast<double *>(c1u)}, 3};
  b[1] = {nz, {v2, c0v, c1v}, {const_cast<double *>(v2), const_cast<double *>(c0v), const_cast<double *>(c1v)}, 3};
  b[2] = {nz + 1, {w2, c0w, c1w},
          {const_cast<double *>(w2), const_cast<double *>(c0w), const_cast<double *>(c1w)}, 3};
  b[3] = {nz + 2, {phi, c0p, c1p},
          {const_cast<double *>(phi), const_cast<double *>(c0p), const_cast<double *>(c1p)}, 3};
  b[4] = {nz + 2, {pres, pres_old, nullptr}, {const_cast<double *>(pres), const_cast<double *>(pres_old), nullptr}, 2};
  return b;
}

}  // namespace

extern "C" {

int tpls_write_backup(const double *u2, const double *v2, const double *w2, const double *conv0_u,
                      const double *conv1_u, const double *conv0_v, const double *conv1_v, const double *conv0_w,
                      const double *conv1_w, const double *pres_old, const double *pres, const double *phi,
                      const double *conv0_phi, const double *conv1_phi, const int *l, const int *m, const int *n,
                      const char *filename) {
  if (!dims_ok(l, m, n)) return TPLS_ERR_ARG;
  const double *all[] = {u2, v2, w2, conv0_u, conv1_u, conv0_v, conv1_v, conv0_w, conv1_w, pres_old, pres, phi,
                         conv0_phi, conv1_phi};
  for (const double *p : all)
    if (!p) return TPLS_ERR_ARG;
  const int nx = *l - 1, ny = *m - 1, nz = *n - 1;
  return write_blocks(filename, nx, ny,
                      main_blocks(nz, u2, v2, w2, conv0_u, conv1_u, conv0_v, conv1_v, conv0_w, conv1_w, pres_old,
                                  pres, phi, conv0_phi, conv1_phi));
}

int tpls_read_backup(double *u2, double *v2, double *w2, double *conv0_u, double *conv1_u, double *conv0_v,
                     double *conv1_v, double *conv0_w, double *conv1_w, double *pres_old, double *pres, double *phi,
                     double *conv0_phi, double *conv1_phi, const int *l, const int *m, const int *n,
                     const char *filename) {
  if (!dims_ok(l, m, n)) return TPLS_ERR_ARG;
  double *all[] = {u2, v2, w2, conv0_u, conv1_u, conv0_v, conv1_v, conv0_w, conv1_w, pres_old, pres, phi,
                   conv0_phi, conv1_phi};
  for (double *p : all)
    if (!p) return TPLS_ERR_ARG;
  const int nx = *l - 1, ny = *m - 1, nz = *n - 1;
  return read_blocks(filename, nx, ny,
                     main_blocks(nz, u2, v2, w2, conv0_u, conv1_u, conv0_v, conv1_v, conv0_w, conv1_w, pres_old,
                                 pres, phi, conv0_phi, conv1_phi));
}

int tpls_write_backup_csf(const double *csf_u0, const double *csf_u1, const double *csf_v0, const double *csf_v1,
                          const double *csf_w0, const double *csf_w1, const int *l, const int *m, const int *n,
                          const char *filename) {
  if (!dims_ok(l, m, n) || !csf_u0 || !csf_u1 || !csf_v0 || !csf_v1 || !csf_w0 || !csf_w1) return TPLS_ERR_ARG;
  const int nx = *l - 1, ny = *m - 1, nz = *n - 1;
  std::vector<Block> b(3);
  b[0] = {nz, {csf_u0, csf_u1, nullptr}, {nullptr, nullptr, nullptr}, 2};
  b[1] = {nz, {csf_v0, csf_v1, nullptr}, {nullptr, nullptr, nullptr}, 2};
  b[2] = {nz + 1, {csf_w0, csf_w1, nullptr}, {nullptr, nullptr, nullptr}, 2};
  return write_blocks(filename, nx, ny, b);
}

int tpls_read_backup_csf(double *csf_u0, double *csf_u1, double *csf_v0, double *csf_v1, double *csf_w0,
                         double *csf_w1, const int *l, const int *m, const int *n, const char *filename) {
  if (!dims_ok(l, m, n) || !csf_u0 || !csf_u1 || !csf_v0 || !csf_v1 || !csf_w0 || !csf_w1) return TPLS_ERR_ARG;
  const int nx = *l - 1, ny = *m - 1, nz = *n - 1;
  std::vector<Block> b(3);
  b[0] = {nz, {nullptr, nullptr, nullptr}, {csf_u0, csf_u1, nullptr}, 2};
  b[1] = {nz, {nullptr, nullptr, nullptr}, {csf_v0, csf_v1, nullptr}, 2};
  b[2] = {nz + 1, {nullptr, nullptr, nullptr}, {csf_w0, csf_w1, nullptr}, 2};
  return read_blocks(filename, nx, ny, b);
}

// --- device state <-> files -------------------------------------------------
}  // extern "C"

namespace {
struct HostState {
  int nx = 0, ny = 0, nz = 0;
  std::vector<double> f[TPLS_F_COUNT];
  double *p(int id) { return f[id].data(); }
};

size_t field_len(int nx, int ny, int nz, int id) {
  const size_t plane = (size_t)(nx + 2) * (size_t)(ny + 2);
  switch (id) {
    case TPLS_F_U2: case TPLS_F_V2: case TPLS_F_CONV0_U: case TPLS_F_CONV1_U: case TPLS_F_CONV0_V:
    case TPLS_F_CONV1_V: case TPLS_F_CSF_U0: case TPLS_F_CSF_U1: case TPLS_F_CSF_V0: case TPLS_F_CSF_V1:
      return plane * (size_t)nz;
    case TPLS_F_W2: case TPLS_F_CONV0_W: case TPLS_F_CONV1_W: case TPLS_F_CSF_W0: case TPLS_F_CSF_W1:
      return plane * (size_t)(nz + 1);
    default:
      return plane * (size_t)(nz + 2);
  }
}

const int kMainFields[] = {TPLS_F_U2, TPLS_F_V2, TPLS_F_W2, TPLS_F_CONV0_U, TPLS_F_CONV1_U, TPLS_F_CONV0_V,
                           TPLS_F_CONV1_V, TPLS_F_CONV0_W, TPLS_F_CONV1_W, TPLS_F_PRES_OLD, TPLS_F_PRES,
                           TPLS_F_PHI2, TPLS_F_CONV0_PHI, TPLS_F_CONV1_PHI};
const int kCsfFields[] = {TPLS_F_CSF_U0, TPLS_F_CSF_U1, TPLS_F_CSF_V0, TPLS_F_CSF_V1, TPLS_F_CSF_W0,
                          TPLS_F_CSF_W1};

int host_state(tpls_ctx *ctx, HostState &h, bool with_csf) {
  int s = tpls_get_dims(ctx, &h.nx, &h.ny, &h.nz);
  if (s) return s;
  for (int id : kMainFields) h.f[id].assign(field_len(h.nx, h.ny, h.nz, id), 0.0);
  if (with_csf)
    for (int id : kCsfFields) h.f[id].assign(field_len(h.nx, h.ny, h.nz, id), 0.0);
  return TPLS_OK;
}
}  // namespace

extern "C" {

int tpls_backup_channel(tpls_ctx *ctx, const char *filename, const char *csf_filename) {
  if (!ctx || !filename) return TPLS_ERR_ARG;
  HostState h;
  int s = host_state(ctx, h, csf_filename != nullptr);
  if (s) return s;
  for (int id : kMainFields)
    if ((s = tpls_get_field(ctx, id, h.p(id)))) return s;
  const int l = h.nx + 1, m = h.ny + 1, n = h.nz + 1;
  s = tpls_write_backup(h.p(TPLS_F_U2), h.p(TPLS_F_V2), h.p(TPLS_F_W2), h.p(TPLS_F_CONV0_U), h.p(TPLS_F_CONV1_U),
                        h.p(TPLS_F_CONV0_V), h.p(TPLS_F_CONV1_V), h.p(TPLS_F_CONV0_W), h.p(TPLS_F_CONV1_W),
                        h.p(TPLS_F_PRES_OLD), h.p(TPLS_F_PRES), h.p(TPLS_F_PHI2), h.p(TPLS_F_CONV0_PHI),
                        h.p(TPLS_F_CONV1_PHI), &l, &m, &n, filename);
  if (s || !csf_filename) return s;
  for (int id : kCsfFields)
    if ((s = tpls_get_field(ctx, id, h.p(id)))) return s;
  return tpls_write_backup_csf(h.p(TPLS_F_CSF_U0), h.p(TPLS_F_CSF_U1), h.p(TPLS_F_CSF_V0), h.p(TPLS_F_CSF_V1),
                               h.p(TPLS_F_CSF_W0), h.p(TPLS_F_CSF_W1), &l, &m, &n, csf_filename);
}

int tpls_dataload_channel(tpls_ctx *ctx, const char *filename, const char *csf_filename) {
  if (!ctx || !filename) return TPLS_ERR_ARG;
  HostState h;
  int s = host_state(ctx, h, csf_filename != nullptr);
  if (s) return s;
  const int l = h.nx + 1, m = h.ny + 1, n = h.nz + 1;
  s = tpls_read_backup(h.p(TPLS_F_U2), h.p(TPLS_F_V2), h.p(TPLS_F_W2), h.p(TPLS_F_CONV0_U), h.p(TPLS_F_CONV1_U),
                       h.p(TPLS_F_CONV0_V), h.p(TPLS_F_CONV1_V), h.p(TPLS_F_CONV0_W), h.p(TPLS_F_CONV1_W),
                       h.p(TPLS_F_PRES_OLD), h.p(TPLS_F_PRES), h.p(TPLS_F_PHI2), h.p(TPLS_F_CONV0_PHI),
                       h.p(TPLS_F_CONV1_PHI), &l, &m, &n, filename);
  if (s) return s;
  if (csf_filename) {
    s = tpls_read_backup_csf(h.p(TPLS_F_CSF_U0), h.p(TPLS_F_CSF_U1), h.p(TPLS_F_CSF_V0), h.p(TPLS_F_CSF_V1),
                             h.p(TPLS_F_CSF_W0), h.p(TPLS_F_CSF_W1), &l, &m, &n, csf_filename);
    if (s) return s;
  }
  // files read completely before the device state is touched
  for (int id : kMainFields)
    if ((s = tpls_set_field(ctx, id, h.p(id)))) return s;
  if (csf_filename)
    for (int id : kCsfFields)
      if ((s = tpls_set_field(ctx, id, h.p(id)))) return s;
  return TPLS_OK;
}

}  // extern "C"
