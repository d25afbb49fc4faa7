// Assembly of the momentum and pressure operators' embedded 7-point rows on
// the GPU. One thread per row computes the row that the CPU setup computes
// (immersed_operators.hpp:1-250, restated in csrc/host/ibm_setup.cpp), with
// the same operations in the same order, so the rows and row scales are
// bitwise the setup's:
//  - neighbours in the reference's insertion order (west, east, south,
//    north, bottom, top), then the diagonal;
//  - cut-cell distances from the ray-circle intersection
//    (common.hpp:262-280);
//  - the row 1-norm summed in the iteration order of the reference's
//    std::unordered_map row (row_scale_sparse, solver_helpers.hpp), and
//    every coefficient scaled by its inverse.
// The functions compile for the host too: with -ffp-contract=off the host
// operations are the same IEEE operations the device intrinsics perform, so
// the row arithmetic is checked against the CPU setup on the CPU.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define IBM_HD __host__ __device__ __forceinline__
#else
#define IBM_HD inline
#endif

namespace ibm {
namespace asmb {

// IEEE double operations, unfused on both sides.
IBM_HD double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
IBM_HD double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
IBM_HD double sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
IBM_HD double dvd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
IBM_HD double sqr(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return sqrt(a);
#endif
}

struct Geo {
  int nx, ny, nz;
  double Lx, Ly, Lz, rho, nu, dt;
  double xcirc, ycirc, Rcirc;
};

// Distance from P along the segment P->S to the cylinder surface, or +inf.
IBM_HD double ray_circle(double xP, double yP, double xS, double yS, const Geo &p) {
  const double inf = __builtin_huge_val();
  const double dx = sub(xS, xP), dy = sub(yS, yP);
  const double a = add(mul(dx, dx), mul(dy, dy));
  if (a <= 0.0) return inf;
  const double ox = sub(xP, p.xcirc), oy = sub(yP, p.ycirc);
  const double b = mul(2.0, add(mul(dx, ox), mul(dy, oy)));
  const double c = sub(add(mul(ox, ox), mul(oy, oy)), mul(p.Rcirc, p.Rcirc));
  const double disc = sub(mul(b, b), mul(mul(4.0, a), c));
  if (disc < 0.0) return inf;
  const double sd = sqr(disc > 0.0 ? disc : 0.0);
  const double t1 = dvd(sub(-b, sd), mul(2.0, a));
  const double t2 = dvd(add(-b, sd), mul(2.0, a));
  double t = inf;
  if (t1 >= 0.0 && t1 <= 1.0) t = t1;
  else if (t2 >= 0.0 && t2 <= 1.0) t = t2;
  if (!(t < inf)) return inf;
  return mul(sqr(a), t);
}

// Iteration order of a 13-bucket std::unordered_map<int, double> filled
// with keys[0..n) in this order (libstdc++: a new bucket's first node goes to
// the list front, a key joins its bucket after the bucket's first node).
IBM_HD void sum_order(const int *keys, int n, int *out) {
  const int kB = 13;
  int nxt[7], before[13];
  int begin = -1;
  for (int b = 0; b < kB; ++b) before[b] = -2;
  for (int x = 0; x < n; ++x) {
    const int b = (int)((unsigned)keys[x] % (unsigned)kB);
    if (before[b] != -2) {
      const int q = before[b];
      if (q == -1) { nxt[x] = begin; begin = x; }
      else { nxt[x] = nxt[q]; nxt[q] = x; }
    } else {
      nxt[x] = begin;
      begin = x;
      if (nxt[x] != -1) before[(int)((unsigned)keys[nxt[x]] % (unsigned)kB)] = x;
      before[b] = -1;
    }
  }
  int m = 0;
  for (int x = begin; x != -1; x = nxt[x]) out[m++] = x;
}

// Slots of the 7-point Struct stencil: C, -x, +x, -y, +y, -z, +z.
enum { C = 0, XM = 1, XP = 2, YM = 3, YP = 4, ZM = 5, ZP = 6 };

struct Row {
  int keys[7], slot[7], n = 0;
  double vals[7];
  IBM_HD void put(int key, double v, int s) { keys[n] = key; vals[n] = v; slot[n] = s; ++n; }
  // Appends the diagonal, writes the row-scaled coefficients, returns the scale.
  IBM_HD double finish(int P, double diag, double *a) {
    put(P, diag, C);
    int ord[7];
    sum_order(keys, n, ord);
    double s = 0.0;
    for (int t = 0; t < n; ++t) s = add(s, fabs(vals[ord[t]]));
    if (s < 1.0e-14) s = 1.0;
    const double sc = dvd(1.0, s);
    for (int t = 0; t < 7; ++t) a[t] = 0.0;
    for (int t = 0; t < n; ++t) a[slot[t]] = mul(sc, vals[t]);
    return sc;
  }
};

struct Coef {
  double dx, dy, dz, cx, cy, cz, at;
};
IBM_HD Coef coef(const Geo &p) {
  Coef c;
  c.dx = dvd(p.Lx, (double)p.nx); c.dy = dvd(p.Ly, (double)p.ny); c.dz = dvd(p.Lz, (double)p.nz);
  c.cx = dvd(p.nu, mul(c.dx, c.dx)); c.cy = dvd(p.nu, mul(c.dy, c.dy)); c.cz = dvd(p.nu, mul(c.dz, c.dz));
  c.at = dvd(p.rho, p.dt);
  return c;
}

IBM_HD long U(const Geo &g, int i, int j, int k) { return ((long)k * g.ny + j) * (g.nx + 1) + i; }
IBM_HD long V(const Geo &g, int i, int j, int k) { return ((long)k * (g.ny + 1) + j) * g.nx + i; }
IBM_HD long W(const Geo &g, int i, int j, int k) { return ((long)k * g.ny + j) * g.nx + i; }

// Row of box row r of field f (0 u, 1 v, 2 w) into a[7]; returns the scale
// and the row's id in *P (0 and an identity row when the face is inactive).
IBM_HD double momentum_row(int f, long r, const Geo &g, const unsigned char *act, const int *id, double *a,
                           int *P) {
  const Coef c = coef(g);
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  int i, j, k;
  if (f == 0) { i = (int)(r % (nx - 1)) + 1; j = (int)((r / (nx - 1)) % ny); k = (int)(r / ((long)(nx - 1) * ny)); }
  else if (f == 1) { i = (int)(r % nx); j = (int)((r / nx) % (ny - 1)) + 1; k = (int)(r / ((long)nx * (ny - 1))); }
  else { i = (int)(r % nx); j = (int)((r / nx) % ny); k = (int)(r / ((long)nx * ny)) + 1; }
  auto face = [&](int ii, int jj, int kk) { return f == 0 ? U(g, ii, jj, kk) : f == 1 ? V(g, ii, jj, kk) : W(g, ii, jj, kk); };
  const long fc = face(i, j, k);
  if (!act[fc]) {
    for (int t = 0; t < 7; ++t) a[t] = 0.0;
    a[C] = 1.0;
    *P = 0;
    return 0.0;
  }
  *P = id[fc];
  Row row;
  double diag = c.at;
  if (f == 0) {
    const double xP = mul((double)i, c.dx), yP = mul((double)(j + 1) - 0.5, c.dy);
    if (i > 1 && act[face(i - 1, j, k)]) { row.put(id[face(i - 1, j, k)], -c.cx, XM); diag = add(diag, c.cx); }
    else if (i == 1) diag = add(diag, c.cx);
    else { const double d = ray_circle(xP, yP, sub(xP, c.dx), yP, g); diag = add(diag, mul(c.cx, dvd(c.dx, d))); }
    if (i < nx - 1 && act[face(i + 1, j, k)]) { row.put(id[face(i + 1, j, k)], -c.cx, XP); diag = add(diag, c.cx); }
    else if (i != nx - 1) { const double d = ray_circle(xP, yP, add(xP, c.dx), yP, g); diag = add(diag, mul(c.cx, dvd(c.dx, d))); }
    if (j > 0 && act[face(i, j - 1, k)]) { row.put(id[face(i, j - 1, k)], -c.cy, YM); diag = add(diag, c.cy); }
    else { const double al = (j == 0) ? dvd(c.dy, mul(0.5, c.dy)) : dvd(c.dy, ray_circle(xP, yP, xP, sub(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    if (j < ny - 1 && act[face(i, j + 1, k)]) { row.put(id[face(i, j + 1, k)], -c.cy, YP); diag = add(diag, c.cy); }
    else { const double al = (j == ny - 1) ? dvd(c.dy, mul(0.5, c.dy)) : dvd(c.dy, ray_circle(xP, yP, xP, add(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    if (k > 0 && act[face(i, j, k - 1)]) { row.put(id[face(i, j, k - 1)], -c.cz, ZM); diag = add(diag, c.cz); }
    else diag = add(diag, mul(2.0, c.cz));
    if (k < nz - 1 && act[face(i, j, k + 1)]) { row.put(id[face(i, j, k + 1)], -c.cz, ZP); diag = add(diag, c.cz); }
    else diag = add(diag, mul(2.0, c.cz));
  } else if (f == 1) {
    const double xP = mul((double)(i + 1) - 0.5, c.dx), yP = mul((double)j, c.dy);
    if (i > 0 && act[face(i - 1, j, k)]) { row.put(id[face(i - 1, j, k)], -c.cx, XM); diag = add(diag, c.cx); }
    else { const double al = (i == 0) ? dvd(c.dx, mul(0.5, c.dx)) : dvd(c.dx, ray_circle(xP, yP, sub(xP, c.dx), yP, g)); diag = add(diag, mul(c.cx, al)); }
    if (i < nx - 1 && act[face(i + 1, j, k)]) { row.put(id[face(i + 1, j, k)], -c.cx, XP); diag = add(diag, c.cx); }
    else if (i != nx - 1) { const double al = dvd(c.dx, ray_circle(xP, yP, add(xP, c.dx), yP, g)); diag = add(diag, mul(c.cx, al)); }
    if (j > 1 && act[face(i, j - 1, k)]) { row.put(id[face(i, j - 1, k)], -c.cy, YM); diag = add(diag, c.cy); }
    else { const double al = (j == 1) ? dvd(c.dy, c.dy) : dvd(c.dy, ray_circle(xP, yP, xP, sub(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    if (j < ny - 1 && act[face(i, j + 1, k)]) { row.put(id[face(i, j + 1, k)], -c.cy, YP); diag = add(diag, c.cy); }
    else { const double al = (j == ny - 1) ? dvd(c.dy, c.dy) : dvd(c.dy, ray_circle(xP, yP, xP, add(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    if (k > 0 && act[face(i, j, k - 1)]) { row.put(id[face(i, j, k - 1)], -c.cz, ZM); diag = add(diag, c.cz); }
    else diag = add(diag, mul(2.0, c.cz));
    if (k < nz - 1 && act[face(i, j, k + 1)]) { row.put(id[face(i, j, k + 1)], -c.cz, ZP); diag = add(diag, c.cz); }
    else diag = add(diag, mul(2.0, c.cz));
  } else {
    const double xP = mul((double)(i + 1) - 0.5, c.dx), yP = mul((double)(j + 1) - 0.5, c.dy);
    if (i > 0 && act[face(i - 1, j, k)]) { row.put(id[face(i - 1, j, k)], -c.cx, XM); diag = add(diag, c.cx); }
    else { const double al = (i == 0) ? dvd(c.dx, mul(0.5, c.dx)) : dvd(c.dx, ray_circle(xP, yP, sub(xP, c.dx), yP, g)); diag = add(diag, mul(c.cx, al)); }
    if (i < nx - 1 && act[face(i + 1, j, k)]) { row.put(id[face(i + 1, j, k)], -c.cx, XP); diag = add(diag, c.cx); }
    else if (i != nx - 1) { const double al = dvd(c.dx, ray_circle(xP, yP, add(xP, c.dx), yP, g)); diag = add(diag, mul(c.cx, al)); }
    if (j > 0 && act[face(i, j - 1, k)]) { row.put(id[face(i, j - 1, k)], -c.cy, YM); diag = add(diag, c.cy); }
    else { const double al = (j == 0) ? dvd(c.dy, mul(0.5, c.dy)) : dvd(c.dy, ray_circle(xP, yP, xP, sub(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    if (j < ny - 1 && act[face(i, j + 1, k)]) { row.put(id[face(i, j + 1, k)], -c.cy, YP); diag = add(diag, c.cy); }
    else { const double al = (j == ny - 1) ? dvd(c.dy, mul(0.5, c.dy)) : dvd(c.dy, ray_circle(xP, yP, xP, add(yP, c.dy), g)); diag = add(diag, mul(c.cy, al)); }
    // the w operator closes the z walls with +cz (immersed_operators.hpp:164-170)
    if (k > 1 && act[face(i, j, k - 1)]) { row.put(id[face(i, j, k - 1)], -c.cz, ZM); diag = add(diag, c.cz); }
    else diag = add(diag, c.cz);
    if (k < nz - 1 && act[face(i, j, k + 1)]) { row.put(id[face(i, j, k + 1)], -c.cz, ZP); diag = add(diag, c.cz); }
    else diag = add(diag, c.cz);
  }
  return row.finish(*P, diag, a);
}

// Inputs of the pressure rows: the cut-cell fractions and the q-face masks
// and ids of the projection (immersed_operators.hpp:179-250).
struct PInputs {
  const unsigned char *fluid;
  const int *id_p;
  const double *beta;
  const double *alpha[3];
  const unsigned char *act_q[3];
  const int *id_q[3];
  int nQu, nQv;
};

// Row of cell c of the sign-flipped pressure operator -D G into a[7]: the
// diagonal is sum over the cell's q-faces of D * G(self) in the iteration
// order of the reference's row map, each neighbour -(D * G(neighbour)).
IBM_HD void pressure_row(long cell, const Geo &g, const PInputs &in, double *a) {
  for (int t = 0; t < 7; ++t) a[t] = 0.0;
  if (!in.fluid[cell]) { a[C] = 1.0; return; }
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int i = (int)(cell % nx), j = (int)((cell / nx) % ny), k = (int)(cell / ((long)nx * ny));
  const double dx = dvd(g.Lx, (double)nx), dy = dvd(g.Ly, (double)ny), dz = dvd(g.Lz, (double)nz);
  const double gx = dvd(1.0, dx), gy = dvd(1.0, dy), gz = dvd(1.0, dz), gout = dvd(2.0, dx);
  const double beta = in.beta[cell];
  auto P = [&](int ii, int jj, int kk) { return ((long)kk * ny + jj) * nx + ii; };
  int keys[6], slot[6], n = 0;
  double dv[6], gs[6], gn[6];
  bool nb[6];
  auto face = [&](int key, double d, int s, double gself, double gnb, bool has) {
    keys[n] = key; dv[n] = d; slot[n] = s; gs[n] = gself; gn[n] = gnb; nb[n] = has; ++n;
  };
  {  // east x-face; the outlet face of the last column has G -2/dx on the cell alone
    const long f = U(g, i + 1, j, k);
    if (in.act_q[0][f]) {
      if (i < nx - 1) face(in.id_q[0][f], dvd(in.alpha[0][f], mul(beta, dx)), XP, -gx, gx, in.id_p[P(i + 1, j, k)] != 0);
      else face(in.id_q[0][f], dvd(in.alpha[0][f], mul(beta, dx)), XP, -gout, 0.0, false);
    }
  }
  if (i > 0) {
    const long f = U(g, i, j, k);
    if (in.act_q[0][f]) face(in.id_q[0][f], dvd(-in.alpha[0][f], mul(beta, dx)), XM, gx, -gx, in.id_p[P(i - 1, j, k)] != 0);
  }
  if (j < ny - 1) {
    const long f = V(g, i, j + 1, k);
    if (in.act_q[1][f]) face(in.nQu + in.id_q[1][f], dvd(in.alpha[1][f], mul(beta, dy)), YP, -gy, gy, in.id_p[P(i, j + 1, k)] != 0);
  }
  if (j > 0) {
    const long f = V(g, i, j, k);
    if (in.act_q[1][f]) face(in.nQu + in.id_q[1][f], dvd(-in.alpha[1][f], mul(beta, dy)), YM, gy, -gy, in.id_p[P(i, j - 1, k)] != 0);
  }
  if (k < nz - 1) {
    const long f = W(g, i, j, k + 1);
    if (in.act_q[2][f]) face(in.nQu + in.nQv + in.id_q[2][f], dvd(in.alpha[2][f], mul(beta, dz)), ZP, -gz, gz, in.id_p[P(i, j, k + 1)] != 0);
  }
  if (k > 0) {
    const long f = W(g, i, j, k);
    if (in.act_q[2][f]) face(in.nQu + in.nQv + in.id_q[2][f], dvd(-in.alpha[2][f], mul(beta, dz)), ZM, gz, -gz, in.id_p[P(i, j, k - 1)] != 0);
  }
  int ord[7];
  sum_order(keys, n, ord);
  double diag = 0.0;
  for (int t = 0; t < n; ++t) diag = add(diag, mul(dv[ord[t]], gs[ord[t]]));
  a[C] = -diag;
  for (int t = 0; t < n; ++t)
    if (nb[t]) a[slot[t]] = -mul(dv[t], gn[t]);
}

}  // namespace asmb
}  // namespace ibm
