// Host-side setup of the immersed-boundary channel case (CPU, once per case).
//
// Builds the cut-cell geometry, masks, ids, the four Struct-embedded 7-point
// operators and the projection CSR in one pass per field, without the
// reference's per-row hash maps. Every floating-point expression is evaluated
// in the same order as the reference so the arrays are bit-identical; the
// two places where the reference's order is the iteration order of a
// std::unordered_map row (row 1-norms in row_scale_sparse,
// immersed_operators.hpp:737-748, and the diagonal of D*G in multiply,
// common.hpp:175-189) use an explicit model of that order (SumOrder below),
// which ibm_host_check_sum_order() verifies against the real container.
//
// Build with -ffp-contract=off: no multiply-add may be fused here.
#include "ibm_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Iteration order of a fresh std::unordered_map<int, double> (libstdc++, GCC
// 11 and later) after inserting up to 13 distinct keys. std::hash<int> is the
// identity. The first insertion sizes the table with the prime policy's
// minimum of 11 buckets, rounded up through its small-prime table to 13, so
// no rehash happens below 14 elements. A key whose bucket already holds nodes
// is linked at the front of that bucket's run; a key whose bucket is empty is
// linked at the front of the whole list.
// ---------------------------------------------------------------------------
struct SumOrder {
  static constexpr int kBuckets = 13;
  // keys[0..n) in insertion order; writes the visiting order (indices) to out.
  static void order(const int *keys, int n, int *out) {
    int nxt[kBuckets];
    int begin = -1;
    int before[kBuckets];  // -2: empty bucket, -1: list head, >=0: node index
    for (int b = 0; b < kBuckets; ++b) before[b] = -2;
    for (int x = 0; x < n; ++x) {
      const int b = bucket(keys[x]);
      if (before[b] != -2) {
        const int p = before[b];
        if (p == -1) { nxt[x] = begin; begin = x; }
        else { nxt[x] = nxt[p]; nxt[p] = x; }
      } else {
        nxt[x] = begin;
        begin = x;
        if (nxt[x] != -1) before[bucket(keys[nxt[x]])] = x;
        before[b] = -1;
      }
    }
    int m = 0;
    for (int x = begin; x != -1; x = nxt[x]) out[m++] = x;
  }
  static int bucket(int key) { return (int)((size_t)key % (size_t)kBuckets); }
};

// ---------------------------------------------------------------------------
// Case storage: named, typed arrays.
// ---------------------------------------------------------------------------
struct Array {
  std::vector<unsigned char> bytes;
  int elem = 0;
};

}  // namespace

struct ibm_case {
  ibm_case_params par;
  ibm_case_counts counts;
  std::map<std::string, Array> arrays;

  template <class T>
  T *alloc(const char *name, size_t n, T init) {
    Array &a = arrays[name];
    a.elem = (int)sizeof(T);
    a.bytes.assign(n * sizeof(T), 0);
    T *p = reinterpret_cast<T *>(a.bytes.data());
    for (size_t i = 0; i < n; ++i) p[i] = init;
    return p;
  }
  template <class T>
  void put(const char *name, const std::vector<T> &v) {
    Array &a = arrays[name];
    a.elem = (int)sizeof(T);
    a.bytes.resize(v.size() * sizeof(T));
    if (!v.empty()) std::memcpy(a.bytes.data(), v.data(), a.bytes.size());
  }
};

namespace {

struct Grid {
  int nx, ny, nz;
  size_t P(int i, int j, int k) const { return ((size_t)k * ny + j) * nx + i; }
  size_t U(int i, int j, int k) const { return ((size_t)k * ny + j) * (nx + 1) + i; }
  size_t V(int i, int j, int k) const { return ((size_t)k * (ny + 1) + j) * nx + i; }
  size_t W(int i, int j, int k) const { return ((size_t)k * ny + j) * nx + i; }
};

// Parabolic inlet profile (common.hpp:240-243), same evaluation order.
inline double inlet_profile(double y, double z, double H, double Um) {
  return 16.0 * Um * y * z * (H - y) * (H - z) / std::pow(H, 4.0);
}

// Distance from P along the segment P->S to the cylinder surface, or +inf
// (common.hpp:262-280), same evaluation order.
inline double ray_circle_distance(double xP, double yP, double xS, double yS, const ibm_case_params &p) {
  const double dx = xS - xP, dy = yS - yP;
  const double a = dx * dx + dy * dy;
  if (a <= 0.0) return std::numeric_limits<double>::infinity();
  const double ox = xP - p.xcirc, oy = yP - p.ycirc;
  const double b = 2.0 * (dx * ox + dy * oy);
  const double c = ox * ox + oy * oy - p.Rcirc * p.Rcirc;
  const double disc = b * b - 4.0 * a * c;
  if (disc < 0.0) return std::numeric_limits<double>::infinity();
  const double sd = std::sqrt(std::max(0.0, disc));
  const double t1 = (-b - sd) / (2.0 * a);
  const double t2 = (-b + sd) / (2.0 * a);
  double t = std::numeric_limits<double>::infinity();
  if (t1 >= 0.0 && t1 <= 1.0) t = t1;
  else if (t2 >= 0.0 && t2 <= 1.0) t = t2;
  if (!std::isfinite(t)) return std::numeric_limits<double>::infinity();
  return std::sqrt(a) * t;
}

// 2-D planar data (the geometry is extruded in z).
struct Plane {
  std::vector<double> beta, alpha_u, alpha_v;           // nx*ny, (nx+1)*ny, nx*(ny+1)
  std::vector<char> fluid, act_u, act_v, act_qu, act_qv;  // same layouts
};

// Open fractions (immersed_geometry.hpp:1-73).
void plane_fractions(const ibm_case_params &p, Plane &pl) {
  const int nx = p.nx, ny = p.ny, ns = p.nsub_beta;
  const double dx = p.Lx / nx, dy = p.Ly / ny;
  std::vector<double> sub((size_t)ns);
  for (int s = 0; s < ns; ++s) sub[(size_t)s] = ((double)s + 0.5) / (double)ns;
  pl.beta.assign((size_t)nx * ny, 0.0);
  const double R2 = p.Rcirc * p.Rcirc;
  for (int i = 0; i < nx; ++i) {
    const double x0 = i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y0 = j * dy;
      int cnt = 0;
      for (int a = 0; a < ns; ++a)
        for (int b = 0; b < ns; ++b) {
          const double xs = x0 + sub[(size_t)a] * dx;
          const double ys = y0 + sub[(size_t)b] * dy;
          const double r2 = (xs - p.xcirc) * (xs - p.xcirc) + (ys - p.ycirc) * (ys - p.ycirc);
          if (r2 > R2) cnt++;
        }
      pl.beta[(size_t)i + (size_t)j * nx] = (double)cnt / (double)(ns * ns);
    }
  }
  pl.alpha_u.assign((size_t)(nx + 1) * ny, 1.0);
  for (int i = 0; i <= nx; ++i) {
    const double x = i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y0 = j * dy, y1 = (j + 1) * dy;
      double val = 1.0;
      if (std::abs(x - p.xcirc) < p.Rcirc) {
        const double h = std::sqrt(std::max(0.0, p.Rcirc * p.Rcirc - (x - p.xcirc) * (x - p.xcirc)));
        const double s0 = p.ycirc - h, s1 = p.ycirc + h;
        const double ov = std::max(0.0, std::min(y1, s1) - std::max(y0, s0));
        val = std::max(0.0, std::min(1.0, 1.0 - ov / dy));
      }
      pl.alpha_u[(size_t)i + (size_t)j * (nx + 1)] = val;
    }
  }
  pl.alpha_v.assign((size_t)nx * (ny + 1), 1.0);
  for (int j = 0; j <= ny; ++j) {
    const double y = j * dy;
    for (int i = 0; i < nx; ++i) {
      const double x0 = i * dx, x1 = (i + 1) * dx;
      double val = 1.0;
      if (std::abs(y - p.ycirc) < p.Rcirc) {
        const double h = std::sqrt(std::max(0.0, p.Rcirc * p.Rcirc - (y - p.ycirc) * (y - p.ycirc)));
        const double s0 = p.xcirc - h, s1 = p.xcirc + h;
        const double ov = std::max(0.0, std::min(x1, s1) - std::max(x0, s0));
        val = std::max(0.0, std::min(1.0, 1.0 - ov / dx));
      }
      pl.alpha_v[(size_t)i + (size_t)j * nx] = val;
    }
  }
}

// Face masks from the fluid-cell mask (immersed_geometry.hpp:75-115).
void plane_masks(const ibm_case_params &p, Plane &pl) {
  const int nx = p.nx, ny = p.ny;
  const double dx = p.Lx / nx, dy = p.Ly / ny, R2 = p.Rcirc * p.Rcirc;
  auto fl = [&](int i, int j) { return pl.fluid[(size_t)i + (size_t)j * nx] != 0; };
  pl.act_u.assign((size_t)(nx + 1) * ny, 0);
  pl.act_qu.assign((size_t)(nx + 1) * ny, 0);
  pl.act_v.assign((size_t)nx * (ny + 1), 0);
  pl.act_qv.assign((size_t)nx * (ny + 1), 0);
  for (int i = 1; i < nx; ++i) {  // interior vertical faces
    const double x = i * dx;
    for (int j = 0; j < ny; ++j) {
      const double y = ((j + 1) - 0.5) * dy;
      const bool outside = ((x - p.xcirc) * (x - p.xcirc) + (y - p.ycirc) * (y - p.ycirc)) > R2;
      const bool adj = fl(i - 1, j) || fl(i, j);
      const size_t s = (size_t)i + (size_t)j * (nx + 1);
      pl.act_u[s] = (char)(outside && adj);
      pl.act_qu[s] = (char)(outside && adj && (pl.alpha_u[s] > p.alpha_tol));
    }
  }
  for (int j = 0; j < ny; ++j) pl.act_qu[(size_t)nx + (size_t)j * (nx + 1)] = (char)fl(nx - 1, j);
  for (int i = 0; i < nx; ++i) {  // interior horizontal faces
    const double x = ((i + 1) - 0.5) * dx;
    for (int j = 1; j < ny; ++j) {
      const double y = j * dy;
      const bool outside = ((x - p.xcirc) * (x - p.xcirc) + (y - p.ycirc) * (y - p.ycirc)) > R2;
      const bool adj = fl(i, j - 1) || fl(i, j);
      const size_t s = (size_t)i + (size_t)j * nx;
      pl.act_v[s] = (char)(outside && adj);
      pl.act_qv[s] = (char)(outside && adj && (pl.alpha_v[s] > p.alpha_tol));
    }
  }
}

// Fluid mask with iterative removal of columns that no open face connects
// (immersed_geometry.hpp:117-160).
int plane_fluid_pruned(const ibm_case_params &p, Plane &pl) {
  const int nx = p.nx, ny = p.ny;
  pl.fluid.assign((size_t)nx * ny, 0);
  for (size_t s = 0; s < pl.fluid.size(); ++s) pl.fluid[s] = (char)(pl.beta[s] > p.beta_tol);
  int pruned = 0;
  for (;;) {
    plane_masks(p, pl);
    std::vector<size_t> drop;
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j) {
        if (!pl.fluid[(size_t)i + (size_t)j * nx]) continue;
        int conn = 0;
        conn += pl.act_qu[(size_t)(i + 1) + (size_t)j * (nx + 1)] ? 1 : 0;  // east (outlet face for i = nx-1)
        if (i > 0) conn += pl.act_qu[(size_t)i + (size_t)j * (nx + 1)] ? 1 : 0;
        if (j < ny - 1) conn += pl.act_qv[(size_t)i + (size_t)(j + 1) * nx] ? 1 : 0;
        if (j > 0) conn += pl.act_qv[(size_t)i + (size_t)j * nx] ? 1 : 0;
        if (conn == 0) drop.push_back((size_t)i + (size_t)j * nx);
      }
    if (drop.empty()) break;
    for (size_t s : drop) pl.fluid[s] = 0;
    pruned += (int)drop.size();
  }
  plane_masks(p, pl);
  return pruned;
}

// Row 1-norm in the reference's summation order (row_scale_sparse).
// keys/vals in insertion order of the reference's row.
inline double row_abs_sum(const int *keys, const double *vals, int n) {
  int ord[SumOrder::kBuckets];
  SumOrder::order(keys, n, ord);
  double s = 0.0;
  for (int t = 0; t < n; ++t) s += std::abs(vals[ord[t]]);
  return s;
}

// Slot numbers of the 7-point Struct stencil (hypre_struct_utils.hpp:9).
enum { S_C = 0, S_XM = 1, S_XP = 2, S_YM = 3, S_YP = 4, S_ZM = 5, S_ZP = 6 };

// One momentum row: neighbours in the reference's insertion order (west,
// east, south, north, bottom, top), then the diagonal; writes the row-scaled
// embedded row and returns the scale.
struct MomRow {
  int keys[7];
  double vals[7];
  int slot[7];
  int n = 0;
  void add(int key, double v, int s) { keys[n] = key; vals[n] = v; slot[n] = s; ++n; }
  double finish(int P, double diag, double *a) {
    add(P, diag, S_C);
    double s = row_abs_sum(keys, vals, n);
    if (s < 1.0e-14) s = 1.0;
    const double sc = 1.0 / s;
    for (int t = 0; t < n; ++t) a[slot[t]] = sc * vals[t];
    return sc;
  }
};

void build_u_operator(const ibm_case_params &p, const Grid &g, const char *act, const int *id, int nU,
                      double *vals, double *scale, double *rhs_bc) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const double dx = p.Lx / nx, dy = p.Ly / ny, dz = p.Lz / nz;
  const double cx = p.nu / (dx * dx), cy = p.nu / (dy * dy), cz = p.nu / (dz * dz), at = p.rho / p.dt;
  (void)nU;
  const size_t nxu = (size_t)nx - 1;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {  // 0-based face index
        double *a = vals + 7 * ((size_t)(i - 1) + nxu * ((size_t)j + (size_t)ny * k));
        const size_t f = g.U(i, j, k);
        if (!act[f]) { a[S_C] = 1.0; continue; }
        const int P = id[f];
        const double xP = i * dx, yP = ((j + 1) - 0.5) * dy, zP = ((k + 1) - 0.5) * dz;
        double diag = at;
        MomRow r;
        if (i > 1 && act[g.U(i - 1, j, k)]) { r.add(id[g.U(i - 1, j, k)], -cx, S_XM); diag += cx; }
        else if (i == 1) { diag += cx; rhs_bc[P] += cx * inlet_profile(yP, zP, p.Ly, 1.0); }
        else { const double d = ray_circle_distance(xP, yP, xP - dx, yP, p); diag += cx * (dx / d); }
        if (i < nx - 1 && act[g.U(i + 1, j, k)]) { r.add(id[g.U(i + 1, j, k)], -cx, S_XP); diag += cx; }
        else if (i != nx - 1) { const double d = ray_circle_distance(xP, yP, xP + dx, yP, p); diag += cx * (dx / d); }
        if (j > 0 && act[g.U(i, j - 1, k)]) { r.add(id[g.U(i, j - 1, k)], -cy, S_YM); diag += cy; }
        else { const double al = (j == 0) ? dy / (0.5 * dy) : dy / ray_circle_distance(xP, yP, xP, yP - dy, p); diag += cy * al; }
        if (j < ny - 1 && act[g.U(i, j + 1, k)]) { r.add(id[g.U(i, j + 1, k)], -cy, S_YP); diag += cy; }
        else { const double al = (j == ny - 1) ? dy / (0.5 * dy) : dy / ray_circle_distance(xP, yP, xP, yP + dy, p); diag += cy * al; }
        if (k > 0 && act[g.U(i, j, k - 1)]) { r.add(id[g.U(i, j, k - 1)], -cz, S_ZM); diag += cz; }
        else diag += 2.0 * cz;
        if (k < nz - 1 && act[g.U(i, j, k + 1)]) { r.add(id[g.U(i, j, k + 1)], -cz, S_ZP); diag += cz; }
        else diag += 2.0 * cz;
        scale[P] = r.finish(P, diag, a);
      }
}

void build_v_operator(const ibm_case_params &p, const Grid &g, const char *act, const int *id,
                      double *vals, double *scale) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const double dx = p.Lx / nx, dy = p.Ly / ny, dz = p.Lz / nz;
  const double cx = p.nu / (dx * dx), cy = p.nu / (dy * dy), cz = p.nu / (dz * dz), at = p.rho / p.dt;
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double *a = vals + 7 * ((size_t)i + (size_t)nx * ((size_t)(j - 1) + (size_t)(ny - 1) * k));
        const size_t f = g.V(i, j, k);
        if (!act[f]) { a[S_C] = 1.0; continue; }
        const int P = id[f];
        const double xP = ((i + 1) - 0.5) * dx, yP = j * dy;
        double diag = at;
        MomRow r;
        if (i > 0 && act[g.V(i - 1, j, k)]) { r.add(id[g.V(i - 1, j, k)], -cx, S_XM); diag += cx; }
        else { const double al = (i == 0) ? dx / (0.5 * dx) : dx / ray_circle_distance(xP, yP, xP - dx, yP, p); diag += cx * al; }
        if (i < nx - 1 && act[g.V(i + 1, j, k)]) { r.add(id[g.V(i + 1, j, k)], -cx, S_XP); diag += cx; }
        else if (i != nx - 1) { const double al = dx / ray_circle_distance(xP, yP, xP + dx, yP, p); diag += cx * al; }
        if (j > 1 && act[g.V(i, j - 1, k)]) { r.add(id[g.V(i, j - 1, k)], -cy, S_YM); diag += cy; }
        else { const double al = (j == 1) ? dy / dy : dy / ray_circle_distance(xP, yP, xP, yP - dy, p); diag += cy * al; }
        if (j < ny - 1 && act[g.V(i, j + 1, k)]) { r.add(id[g.V(i, j + 1, k)], -cy, S_YP); diag += cy; }
        else { const double al = (j == ny - 1) ? dy / dy : dy / ray_circle_distance(xP, yP, xP, yP + dy, p); diag += cy * al; }
        if (k > 0 && act[g.V(i, j, k - 1)]) { r.add(id[g.V(i, j, k - 1)], -cz, S_ZM); diag += cz; }
        else diag += 2.0 * cz;
        if (k < nz - 1 && act[g.V(i, j, k + 1)]) { r.add(id[g.V(i, j, k + 1)], -cz, S_ZP); diag += cz; }
        else diag += 2.0 * cz;
        scale[P] = r.finish(P, diag, a);
      }
}

void build_w_operator(const ibm_case_params &p, const Grid &g, const char *act, const int *id,
                      double *vals, double *scale) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const double dx = p.Lx / nx, dy = p.Ly / ny, dz = p.Lz / nz;
  const double cx = p.nu / (dx * dx), cy = p.nu / (dy * dy), cz = p.nu / (dz * dz), at = p.rho / p.dt;
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        double *a = vals + 7 * ((size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (k - 1)));
        const size_t f = g.W(i, j, k);
        if (!act[f]) { a[S_C] = 1.0; continue; }
        const int P = id[f];
        const double xP = ((i + 1) - 0.5) * dx, yP = ((j + 1) - 0.5) * dy;
        double diag = at;
        MomRow r;
        if (i > 0 && act[g.W(i - 1, j, k)]) { r.add(id[g.W(i - 1, j, k)], -cx, S_XM); diag += cx; }
        else { const double al = (i == 0) ? dx / (0.5 * dx) : dx / ray_circle_distance(xP, yP, xP - dx, yP, p); diag += cx * al; }
        if (i < nx - 1 && act[g.W(i + 1, j, k)]) { r.add(id[g.W(i + 1, j, k)], -cx, S_XP); diag += cx; }
        else if (i != nx - 1) { const double al = dx / ray_circle_distance(xP, yP, xP + dx, yP, p); diag += cx * al; }
        if (j > 0 && act[g.W(i, j - 1, k)]) { r.add(id[g.W(i, j - 1, k)], -cy, S_YM); diag += cy; }
        else { const double al = (j == 0) ? dy / (0.5 * dy) : dy / ray_circle_distance(xP, yP, xP, yP - dy, p); diag += cy * al; }
        if (j < ny - 1 && act[g.W(i, j + 1, k)]) { r.add(id[g.W(i, j + 1, k)], -cy, S_YP); diag += cy; }
        else { const double al = (j == ny - 1) ? dy / (0.5 * dy) : dy / ray_circle_distance(xP, yP, xP, yP + dy, p); diag += cy * al; }
        // The w operator closes the z walls with +cz (not +2cz): immersed_operators.hpp:164-170.
        if (k > 1 && act[g.W(i, j, k - 1)]) { r.add(id[g.W(i, j, k - 1)], -cz, S_ZM); diag += cz; }
        else diag += cz;
        if (k < nz - 1 && act[g.W(i, j, k + 1)]) { r.add(id[g.W(i, j, k + 1)], -cz, S_ZP); diag += cz; }
        else diag += cz;
        scale[P] = r.finish(P, diag, a);
      }
}

int max_id(const std::vector<int> &id) { return id.empty() ? 0 : *std::max_element(id.begin(), id.end()); }

void number_active(const char *mask, size_t n, std::vector<int> &id) {
  id.assign(n, 0);
  int c = 0;
  for (size_t t = 0; t < n; ++t)
    if (mask[t]) id[t] = ++c;
}

}  // namespace

extern "C" {

void ibm_case_params_default(ibm_case_params *p) {
  p->nx = 32; p->ny = 12; p->nz = 12;
  p->Lx = 2.2; p->Ly = 0.41; p->Lz = 0.41;
  p->rho = 1.0; p->nu = 1.0e-3; p->Um = 0.45; p->dt = 2.0e-3;
  p->nsub_beta = 10; p->beta_tol = 1.0e-8; p->alpha_tol = 1.0e-10;
  p->xcirc = 0.2; p->ycirc = 0.2; p->Rcirc = 0.05;
}

int ibm_case_build(const ibm_case_params *pp, ibm_case **out) {
  if (!pp || !out) return -1;
  const ibm_case_params p = *pp;
  if (p.nx < 3 || p.ny < 3 || p.nz < 3 || p.nsub_beta < 1) return -1;
  const double cells = (double)p.nx * p.ny * p.nz;
  if (cells * 7.0 > 2.0e9) return -1;  // 1-based int32 ids and CSR offsets must fit
  ibm_case *c = new ibm_case();
  c->par = p;
  const Grid g{p.nx, p.ny, p.nz};
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const double dx = p.Lx / nx, dy = p.Ly / ny, dz = p.Lz / nz;

  Plane pl;
  plane_fractions(p, pl);
  const int pruned = plane_fluid_pruned(p, pl);

  // z-extrusion (main.cu:33-71)
  const size_t NP = (size_t)nx * ny * nz, NU = (size_t)(nx + 1) * ny * nz, NV = (size_t)nx * (ny + 1) * nz,
               NW = (size_t)nx * ny * (nz + 1);
  double *beta_p = c->alloc<double>("beta_p", NP, 0.0);
  double *alpha_u = c->alloc<double>("alpha_u", NU, 0.0);
  double *alpha_v = c->alloc<double>("alpha_v", NV, 0.0);
  double *alpha_w = c->alloc<double>("alpha_w", NW, 1.0);
  char *fluid_p = (char *)c->alloc<unsigned char>("fluid_p", NP, 0);
  char *act_u = (char *)c->alloc<unsigned char>("active_u", NU, 0);
  char *act_v = (char *)c->alloc<unsigned char>("active_v", NV, 0);
  char *act_w = (char *)c->alloc<unsigned char>("active_w", NW, 0);
  char *act_qu = (char *)c->alloc<unsigned char>("active_qu", NU, 0);
  char *act_qv = (char *)c->alloc<unsigned char>("active_qv", NV, 0);
  char *act_qw = (char *)c->alloc<unsigned char>("active_qw", NW, 0);
  for (int k = 0; k < nz; ++k) {
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t s = (size_t)i + (size_t)j * nx;
        beta_p[g.P(i, j, k)] = pl.beta[s];
        fluid_p[g.P(i, j, k)] = pl.fluid[s];
      }
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const size_t s = (size_t)i + (size_t)j * (nx + 1), f = g.U(i, j, k);
        alpha_u[f] = pl.alpha_u[s]; act_u[f] = pl.act_u[s]; act_qu[f] = pl.act_qu[s];
      }
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t s = (size_t)i + (size_t)j * nx, f = g.V(i, j, k);
        alpha_v[f] = pl.alpha_v[s]; act_v[f] = pl.act_v[s]; act_qv[f] = pl.act_qv[s];
      }
  }
  // A w face is active when a fluid cell lies on either side in z; the masks
  // are z-invariant, so this is the column's fluid flag on every level.
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const bool adj = (k > 0 && fluid_p[g.P(i, j, k - 1)]) || (k < nz && fluid_p[g.P(i, j, k)]);
        act_w[g.W(i, j, k)] = (char)adj;
        act_qw[g.W(i, j, k)] = (char)adj;
      }

  std::vector<int> id_u, id_v, id_w, id_p, id_qu, id_qv, id_qw;
  number_active(act_u, NU, id_u); number_active(act_v, NV, id_v); number_active(act_w, NW, id_w);
  number_active(fluid_p, NP, id_p); number_active(act_qu, NU, id_qu); number_active(act_qv, NV, id_qv);
  number_active(act_qw, NW, id_qw);
  const int nU = max_id(id_u), nV = max_id(id_v), nW = max_id(id_w), nP = max_id(id_p);
  const int nQu = max_id(id_qu), nQv = max_id(id_qv), nQw = max_id(id_qw);
  c->counts = ibm_case_counts{nU, nV, nW, nP, nQu, nQv, nQw, pruned};

  // Momentum operators, row-scaled and embedded (immersed_operators.hpp:1-177,
  // 737-748; solver_helpers.hpp:51-84, 227-295).
  double *Au = c->alloc<double>("Au_vals", (size_t)(nx - 1) * ny * nz * 7, 0.0);
  double *Av = c->alloc<double>("Av_vals", (size_t)nx * (ny - 1) * nz * 7, 0.0);
  double *Aw = c->alloc<double>("Aw_vals", (size_t)nx * ny * (nz - 1) * 7, 0.0);
  double *scale_u = c->alloc<double>("scale_u", (size_t)nU + 1, 1.0);
  double *scale_v = c->alloc<double>("scale_v", (size_t)nV + 1, 1.0);
  double *scale_w = c->alloc<double>("scale_w", (size_t)nW + 1, 1.0);
  double *rhs_u_bc = c->alloc<double>("rhs_u_bc", (size_t)nU + 1, 0.0);
  c->alloc<double>("rhs_v_bc", (size_t)nV + 1, 0.0);
  c->alloc<double>("rhs_w_bc", (size_t)nW + 1, 0.0);
  build_u_operator(p, g, act_u, id_u.data(), nU, Au, scale_u, rhs_u_bc);
  build_v_operator(p, g, act_v, id_v.data(), Av, scale_v);
  build_w_operator(p, g, act_w, id_w.data(), Aw, scale_w);

  // Projection operators (immersed_operators.hpp:179-287). D rows are built
  // in the reference's insertion order east, west, north, south, top, bottom.
  const double ginv_x = 1.0 / dx, ginv_y = 1.0 / dy, ginv_z = 1.0 / dz, gout = 2.0 / dx;
  std::vector<int> Drow((size_t)nP + 1, 0), Dcol;
  std::vector<double> Dval;
  Dcol.reserve((size_t)nP * 6); Dval.reserve((size_t)nP * 6);
  double *div_bc = c->alloc<double>("div_bc_unit", (size_t)nP + 1, 0.0);
  double *Ap = c->alloc<double>("Ap_vals", NP * 7, 0.0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t cell = g.P(i, j, k);
        double *a = Ap + 7 * cell;
        if (!fluid_p[cell]) { a[S_C] = 1.0; continue; }
        const int row = id_p[cell];
        const double beta = beta_p[cell];
        int keys[6], slot[6];
        double dv[6], gself[6], gnb[6];
        bool has_nb[6];
        int n = 0;
        auto face = [&](int key, double dval, int s, double gs, double gn, bool nb) {
          keys[n] = key; dv[n] = dval; slot[n] = s; gself[n] = gs; gnb[n] = gn; has_nb[n] = nb; ++n;
        };
        // east x-face (the outlet face for the last column: G row -2/dx on the cell alone)
        {
          const size_t f = g.U(i + 1, j, k);
          if (act_qu[f]) {
            if (i < nx - 1) face(id_qu[f], alpha_u[f] / (beta * dx), S_XP, -ginv_x, ginv_x, id_p[g.P(i + 1, j, k)] != 0);
            else face(id_qu[f], alpha_u[f] / (beta * dx), S_XP, -gout, 0.0, false);
          }
        }
        if (i > 0) {
          const size_t f = g.U(i, j, k);
          if (act_qu[f]) face(id_qu[f], -alpha_u[f] / (beta * dx), S_XM, ginv_x, -ginv_x, id_p[g.P(i - 1, j, k)] != 0);
        } else {
          const double y = ((j + 1) - 0.5) * dy, z = ((k + 1) - 0.5) * dz;
          div_bc[row] -= inlet_profile(y, z, p.Ly, p.Um) / (beta * dx);
        }
        if (j < ny - 1) {
          const size_t f = g.V(i, j + 1, k);
          if (act_qv[f]) face(nQu + id_qv[f], alpha_v[f] / (beta * dy), S_YP, -ginv_y, ginv_y, id_p[g.P(i, j + 1, k)] != 0);
        }
        if (j > 0) {
          const size_t f = g.V(i, j, k);
          if (act_qv[f]) face(nQu + id_qv[f], -alpha_v[f] / (beta * dy), S_YM, ginv_y, -ginv_y, id_p[g.P(i, j - 1, k)] != 0);
        }
        if (k < nz - 1) {
          const size_t f = g.W(i, j, k + 1);
          if (act_qw[f]) face(nQu + nQv + id_qw[f], alpha_w[f] / (beta * dz), S_ZP, -ginv_z, ginv_z, id_p[g.P(i, j, k + 1)] != 0);
        }
        if (k > 0) {
          const size_t f = g.W(i, j, k);
          if (act_qw[f]) face(nQu + nQv + id_qw[f], -alpha_w[f] / (beta * dz), S_ZM, ginv_z, -ginv_z, id_p[g.P(i, j, k - 1)] != 0);
        }
        // diagonal of D*G accumulated in the reference row's iteration order
        int ord[SumOrder::kBuckets];
        SumOrder::order(keys, n, ord);
        double diag = 0.0;
        for (int t = 0; t < n; ++t) diag += dv[ord[t]] * gself[ord[t]];
        a[S_C] = -diag;
        for (int t = 0; t < n; ++t)
          if (has_nb[t]) a[slot[t]] = -(dv[t] * gnb[t]);
        // CSR row of D, columns ascending
        int idx[6];
        for (int t = 0; t < n; ++t) idx[t] = t;
        std::sort(idx, idx + n, [&](int x, int y) { return keys[x] < keys[y]; });
        for (int t = 0; t < n; ++t) { Dcol.push_back(keys[idx[t]]); Dval.push_back(dv[idx[t]]); }
        Drow[(size_t)row] = (int)Dcol.size();
      }
  // Rows were produced in cell order, which is id order, so Drow[row] holds
  // each row's end offset: a 1-based CSR rowptr.
  c->put("D_rowptr", Drow);
  c->put("D_col", Dcol);
  c->put("D_val", Dval);

  // G rows (immersed_operators.hpp:251-282), one per q face, columns ascending.
  const int nQ = nQu + nQv + nQw;
  std::vector<int> Grow((size_t)nQ + 1, 0), Gcol;
  std::vector<double> Gval;
  std::vector<int> gcnt((size_t)nQ + 1, 0);
  std::vector<int> gc0((size_t)nQ + 1, 0), gc1((size_t)nQ + 1, 0);
  std::vector<double> gv0((size_t)nQ + 1, 0.0), gv1((size_t)nQ + 1, 0.0);
  auto gput = [&](int row, int col, double v) {
    if (col < 1) return;
    if (gcnt[(size_t)row] == 0) { gc0[(size_t)row] = col; gv0[(size_t)row] = v; }
    else { gc1[(size_t)row] = col; gv1[(size_t)row] = v; }
    gcnt[(size_t)row]++;
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 1; i < nx; ++i) {
        const size_t f = g.U(i, j, k);
        if (!act_qu[f]) continue;
        gput(id_qu[f], id_p[g.P(i - 1, j, k)], -ginv_x);
        gput(id_qu[f], id_p[g.P(i, j, k)], ginv_x);
      }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) {
      const size_t f = g.U(nx, j, k);
      if (!act_qu[f]) continue;
      gput(id_qu[f], id_p[g.P(nx - 1, j, k)], -gout);
    }
  for (int k = 0; k < nz; ++k)
    for (int j = 1; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t f = g.V(i, j, k);
        if (!act_qv[f]) continue;
        gput(nQu + id_qv[f], id_p[g.P(i, j - 1, k)], -ginv_y);
        gput(nQu + id_qv[f], id_p[g.P(i, j, k)], ginv_y);
      }
  for (int k = 1; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t f = g.W(i, j, k);
        if (!act_qw[f]) continue;
        gput(nQu + nQv + id_qw[f], id_p[g.P(i, j, k - 1)], -ginv_z);
        gput(nQu + nQv + id_qw[f], id_p[g.P(i, j, k)], ginv_z);
      }
  for (int r = 1; r <= nQ; ++r) {
    const size_t s = (size_t)r;
    if (gcnt[s] == 1) { Gcol.push_back(gc0[s]); Gval.push_back(gv0[s]); }
    else if (gcnt[s] == 2) {
      if (gc0[s] < gc1[s]) { Gcol.push_back(gc0[s]); Gval.push_back(gv0[s]); Gcol.push_back(gc1[s]); Gval.push_back(gv1[s]); }
      else { Gcol.push_back(gc1[s]); Gval.push_back(gv1[s]); Gcol.push_back(gc0[s]); Gval.push_back(gv0[s]); }
    }
    Grow[s] = (int)Gcol.size();
  }
  c->put("G_rowptr", Grow);
  c->put("G_col", Gcol);
  c->put("G_val", Gval);

  c->put("id_u", id_u); c->put("id_v", id_v); c->put("id_w", id_w); c->put("id_p", id_p);
  c->put("id_qu", id_qu); c->put("id_qv", id_qv); c->put("id_qw", id_qw);

  double *uin = c->alloc<double>("uin", (size_t)ny * nz, 0.0);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      uin[(size_t)j + (size_t)ny * k] = inlet_profile((j + 0.5) * dy, (k + 0.5) * dz, p.Ly, p.Um);
  *out = c;
  return 0;
}

void ibm_case_free(ibm_case *c) { delete c; }

int ibm_case_get_counts(const ibm_case *c, ibm_case_counts *out) {
  if (!c || !out) return -1;
  *out = c->counts;
  return 0;
}

long ibm_case_array_bytes(const ibm_case *c, const char *name, int *elem_size) {
  if (!c || !name) return -1;
  auto it = c->arrays.find(name);
  if (it == c->arrays.end()) return -1;
  if (elem_size) *elem_size = it->second.elem;
  return (long)it->second.bytes.size();
}

const void *ibm_case_array(const ibm_case *c, const char *name) {
  if (!c || !name) return nullptr;
  auto it = c->arrays.find(name);
  if (it == c->arrays.end()) return nullptr;
  return it->second.bytes.data();
}

// File layout: magic "IBMCASE\0", u32 version, the ibm_case_params bytes,
// the counts, u32 array count, then per array: u32 name length, name,
// i32 element size, u64 byte count, bytes. Little-endian host order.
static const char kMagic[8] = {'I', 'B', 'M', 'C', 'A', 'S', 'E', 0};
static const uint32_t kVersion = 1;

int ibm_case_save(const ibm_case *c, const char *path) {
  if (!c || !path) return -1;
  const std::string tmp = std::string(path) + ".tmp";
  std::FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return -2;
  bool ok = std::fwrite(kMagic, 1, 8, f) == 8;
  ok = ok && std::fwrite(&kVersion, sizeof(kVersion), 1, f) == 1;
  ok = ok && std::fwrite(&c->par, sizeof(c->par), 1, f) == 1;
  ok = ok && std::fwrite(&c->counts, sizeof(c->counts), 1, f) == 1;
  const uint32_t na = (uint32_t)c->arrays.size();
  ok = ok && std::fwrite(&na, sizeof(na), 1, f) == 1;
  for (const auto &kv : c->arrays) {
    const uint32_t ln = (uint32_t)kv.first.size();
    const int32_t es = kv.second.elem;
    const uint64_t nb = kv.second.bytes.size();
    ok = ok && std::fwrite(&ln, sizeof(ln), 1, f) == 1 && std::fwrite(kv.first.data(), 1, ln, f) == ln;
    ok = ok && std::fwrite(&es, sizeof(es), 1, f) == 1 && std::fwrite(&nb, sizeof(nb), 1, f) == 1;
    ok = ok && (nb == 0 || std::fwrite(kv.second.bytes.data(), 1, nb, f) == nb);
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) { std::remove(tmp.c_str()); return -2; }
  return std::rename(tmp.c_str(), path) == 0 ? 0 : -2;
}

int ibm_case_load(const ibm_case_params *p, const char *path, ibm_case **out) {
  if (!p || !path || !out) return -1;
  *out = nullptr;
  std::FILE *f = std::fopen(path, "rb");
  if (!f) return 1;
  char magic[8];
  uint32_t ver = 0;
  ibm_case_params fp;
  std::unique_ptr<ibm_case> c(new ibm_case());
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0;
  ok = ok && std::fread(&ver, sizeof(ver), 1, f) == 1 && ver == kVersion;
  ok = ok && std::fread(&fp, sizeof(fp), 1, f) == 1 && std::memcmp(&fp, p, sizeof(fp)) == 0;
  if (!ok) { std::fclose(f); return 1; }
  c->par = fp;
  uint32_t na = 0;
  ok = std::fread(&c->counts, sizeof(c->counts), 1, f) == 1 && std::fread(&na, sizeof(na), 1, f) == 1;
  for (uint32_t a = 0; ok && a < na; ++a) {
    uint32_t ln = 0;
    int32_t es = 0;
    uint64_t nb = 0;
    ok = std::fread(&ln, sizeof(ln), 1, f) == 1 && ln < 256;
    std::string name(ok ? ln : 0, '\0');
    ok = ok && std::fread(&name[0], 1, ln, f) == ln;
    ok = ok && std::fread(&es, sizeof(es), 1, f) == 1 && std::fread(&nb, sizeof(nb), 1, f) == 1;
    if (!ok) break;
    Array &arr = c->arrays[name];
    arr.elem = es;
    arr.bytes.resize((size_t)nb);
    ok = nb == 0 || std::fread(arr.bytes.data(), 1, (size_t)nb, f) == nb;
  }
  std::fclose(f);
  if (!ok) return -2;
  *out = c.release();
  return 0;
}

int ibm_case_build_cached(const ibm_case_params *p, const char *path, ibm_case **out) {
  const int rc = ibm_case_load(p, path, out);
  if (rc == 0) return 0;
  const int b = ibm_case_build(p, out);
  if (b != 0) return b;
  ibm_case_save(*out, path);  // a cache that cannot be written is not an error
  return 0;
}

int ibm_write_vtk(const char *path, const double *u, const double *v, const double *w, const double *p,
                  const uint8_t *fluid_p, int nx, int ny, int nz, double Lx, double Ly, double Lz) {
  if (!path || !u || !v || !w || !p || !fluid_p || nx < 1 || ny < 1 || nz < 1) return -1;
  std::FILE *f = std::fopen(path, "w");
  if (!f) return -2;
  const long sy = nx + 1, sz = (long)(nx + 1) * ny;              // u strides
  const long vy = nx, vz = (long)nx * (ny + 1);                   // v strides
  const long wz = (long)nx * ny;                                  // w plane
  std::fprintf(f, "# vtk DataFile Version 3.0\n3D immersed cylinder MAC cell-centered\nASCII\n"
                  "DATASET STRUCTURED_POINTS\nDIMENSIONS %d %d %d\nORIGIN 0 0 0\nSPACING %.16e %.16e %.16e\n"
                  "CELL_DATA %d\n", nx + 1, ny + 1, nz + 1, Lx / nx, Ly / ny, Lz / nz, nx * ny * nz);
  std::fprintf(f, "SCALARS ux double 1\nLOOKUP_TABLE default\n");
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long a = k * sz + j * sy + i;
        std::fprintf(f, "%.16e\n", 0.5 * (u[a] + u[a + 1]));
      }
  std::fprintf(f, "SCALARS uy double 1\nLOOKUP_TABLE default\n");
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const long a = k * vz + j * vy + i;
        std::fprintf(f, "%.16e\n", 0.5 * (v[a] + v[a + vy]));
      }
  std::fprintf(f, "SCALARS uz double 1\nLOOKUP_TABLE default\n");
  for (long c = 0; c < (long)nx * ny * nz; ++c) std::fprintf(f, "%.16e\n", 0.5 * (w[c] + w[c + wz]));
  std::fprintf(f, "SCALARS pressure double 1\nLOOKUP_TABLE default\n");
  for (long c = 0; c < (long)nx * ny * nz; ++c) std::fprintf(f, "%.16e\n", p[c]);
  std::fprintf(f, "SCALARS fluid_mask int 1\nLOOKUP_TABLE default\n");
  for (long c = 0; c < (long)nx * ny * nz; ++c) std::fprintf(f, "%d\n", fluid_p[c] ? 1 : 0);
  const int bad = std::ferror(f);
  return (std::fclose(f) == 0 && !bad) ? 0 : -2;
}

int ibm_vtk_step_name(const char *base, int step, char *out, int len) {
  if (!base || !out || len < 1) return -1;
  const std::string b(base);
  const size_t dot = b.find_last_of('.');
  const std::string stem = dot == std::string::npos ? b : b.substr(0, dot);
  const std::string ext = dot == std::string::npos ? std::string() : b.substr(dot);
  char num[32];
  std::snprintf(num, sizeof(num), "_%06d", step);
  const std::string name = stem + num + ext;
  std::snprintf(out, (size_t)len, "%s", name.c_str());
  return (int)name.size();
}

int ibm_host_check_sum_order(int ntrials, unsigned seed) {
  std::mt19937 rng(seed);
  int bad = 0;
  for (int t = 0; t < ntrials; ++t) {
    const int n = 1 + (int)(rng() % 7);
    const int base = 1 + (int)(rng() % 100000);
    int keys[7];
    for (int a = 0; a < n; ++a) {
      for (;;) {
        const int k = base + (int)(rng() % 5000);
        bool dup = false;
        for (int b = 0; b < a; ++b) dup |= (keys[b] == k);
        if (!dup) { keys[a] = k; break; }
      }
    }
    std::unordered_map<int, double> m;
    for (int a = 0; a < n; ++a) m[keys[a]] += 1.0;
    int ord[SumOrder::kBuckets];
    SumOrder::order(keys, n, ord);
    int pos = 0;
    bool ok = true;
    for (const auto &kv : m) ok &= (kv.first == keys[ord[pos++]]);
    bad += ok ? 0 : 1;
  }
  return bad;
}

}  // extern "C"
