// Test-only checker: compiles the reference's own CPU setup code
// (immersed_geometry.hpp, immersed_operators.hpp, solver_helpers.hpp) from its
// original location and exposes it through a small extern "C" surface, so the
// tests can compare this repository's host assembly and CPU dense-op oracle
// against the reference itself. Nothing in the product links this file.
//
// The orchestration below follows the order of the reference's setup
// (main.cu:20-116): 2-D fractions, mask pruning, z-extrusion, 1-based ids,
// operator assembly, row scaling, Ap sign flip, row-major embedding, CSR build.
#include "common.hpp"
#include "immersed_geometry.hpp"
#include "immersed_operators.hpp"
#include "hypre_struct_utils.hpp"
#include "gpu_dense_ops.hpp"
#include "solver_helpers.hpp"

#include <map>
#include <string>

namespace {

struct RefArray {
  std::vector<unsigned char> bytes;
  int elem = 0;
};

struct RefCase {
  Params par;
  std::map<std::string, RefArray> arrays;
  template <class T>
  void put(const char *name, const std::vector<T> &v) {
    RefArray a;
    a.elem = (int)sizeof(T);
    a.bytes.resize(v.size() * sizeof(T));
    if (!v.empty()) std::memcpy(a.bytes.data(), v.data(), a.bytes.size());
    arrays[name] = std::move(a);
  }
  void put_csr(const char *prefix, const SparseMatrix &A) {
    std::vector<int> rowptr((size_t)A.nrows + 1, 0), col;
    std::vector<double> val;
    for (int i = 0; i < A.nrows; ++i) {
      std::vector<std::pair<int, double>> row(A.rows[(size_t)i].begin(), A.rows[(size_t)i].end());
      std::sort(row.begin(), row.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
      for (const auto &kv : row) { col.push_back(kv.first); val.push_back(kv.second); }
      rowptr[(size_t)i + 1] = (int)col.size();
    }
    std::string p(prefix);
    put((p + "_rowptr").c_str(), rowptr);
    put((p + "_col").c_str(), col);
    put((p + "_val").c_str(), val);
  }
};

}  // namespace

extern "C" {

// Geometry / physics subset of the reference Params (common.hpp:45-66).
struct ref_case_params {
  int nx, ny, nz;
  double Lx, Ly, Lz, rho, nu, Um, dt;
  int nsub_beta;
  double beta_tol, alpha_tol, xcirc, ycirc, Rcirc;
};

void *ref_case_build(const ref_case_params *cp) {
  RefCase *rc = new RefCase();
  Params &par = rc->par;
  par.nx = cp->nx; par.ny = cp->ny; par.nz = cp->nz;
  par.Lx = cp->Lx; par.Ly = cp->Ly; par.Lz = cp->Lz;
  par.rho = cp->rho; par.nu = cp->nu; par.Um = cp->Um; par.dt = cp->dt;
  par.nsub_beta = cp->nsub_beta; par.beta_tol = cp->beta_tol; par.alpha_tol = cp->alpha_tol;
  par.xcirc = cp->xcirc; par.ycirc = cp->ycirc; par.Rcirc = cp->Rcirc;
  const int nx = par.nx, ny = par.ny, nz = par.nz;
  const double dy = par.Ly / ny, dz = par.Lz / nz;

  std::vector<double> beta2d, alpha_u2d, alpha_v2d;
  compute_pressure_area_fractions_2d(beta2d, par);
  compute_vertical_face_open_fractions_2d(alpha_u2d, par);
  compute_horizontal_face_open_fractions_2d(alpha_v2d, par);
  std::vector<char> fluid2d, active_u2d, active_v2d, active_qu2d, active_qv2d;
  std::vector<std::pair<int, int>> pruned_cols;
  int n_pruned = build_and_prune_2d_masks(fluid2d, active_u2d, active_v2d, active_qu2d, active_qv2d,
                                          beta2d, alpha_u2d, alpha_v2d, par, pruned_cols);

  const size_t NP = (size_t)nx * ny * nz, NU = (size_t)(nx + 1) * ny * nz,
               NV = (size_t)nx * (ny + 1) * nz, NW = (size_t)nx * ny * (nz + 1);
  std::vector<double> beta_p(NP, 0.0), alpha_u(NU, 0.0), alpha_v(NV, 0.0), alpha_w(NW, 1.0);
  std::vector<char> fluid_p(NP, 0), active_u(NU, 0), active_v(NV, 0), active_w(NW, 0),
      active_qu(NU, 0), active_qv(NV, 0), active_qw(NW, 0);
  for (int k = 1; k <= nz; ++k) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t id = idxP3(i - 1, j - 1, k - 1, nx, ny);
        beta_p[id] = beta2d[(size_t)id2_flat(i, j, nx) - 1];
        fluid_p[id] = fluid2d[(size_t)id2_flat(i, j, nx) - 1];
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx + 1; ++i) {
        size_t id = idxU3(i - 1, j - 1, k - 1, nx, ny);
        size_t s = (size_t)(i - 1) + (size_t)(j - 1) * (size_t)(nx + 1);
        alpha_u[id] = alpha_u2d[s]; active_u[id] = active_u2d[s]; active_qu[id] = active_qu2d[s];
      }
    for (int j = 1; j <= ny + 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t id = idxV3(i - 1, j - 1, k - 1, nx, ny);
        size_t s = (size_t)(i - 1) + (size_t)(j - 1) * (size_t)nx;
        alpha_v[id] = alpha_v2d[s]; active_v[id] = active_v2d[s]; active_qv[id] = active_qv2d[s];
      }
  }
  for (int kw = 1; kw <= nz + 1; ++kw)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        bool adj = (kw > 1 && fluid3_at(fluid_p, i, j, kw - 1, nx, ny)) || (kw <= nz && fluid3_at(fluid_p, i, j, kw, nx, ny));
        size_t id = idxW3(i - 1, j - 1, kw - 1, nx, ny);
        active_w[id] = (char)adj; active_qw[id] = (char)adj;
      }
  std::vector<int> id_u, id_v, id_w, id_p, id_qu, id_qv, id_qw;
  build_indices(active_u, id_u); build_indices(active_v, id_v); build_indices(active_w, id_w);
  build_indices(fluid_p, id_p); build_indices(active_qu, id_qu); build_indices(active_qv, id_qv);
  build_indices(active_qw, id_qw);

  SparseMatrix Au0, Av0, Aw0, Dproj, Gproj, Ap0;
  std::vector<double> rhs_u_bc_unit, rhs_v_bc, rhs_w_bc, div_bc_unit;
  build_u_diffusion_3d_immersed(Au0, rhs_u_bc_unit, active_u, id_u, par);
  build_v_diffusion_3d_immersed(Av0, rhs_v_bc, active_v, id_v, par);
  build_w_diffusion_3d_immersed(Aw0, rhs_w_bc, active_w, id_w, par);
  build_projection_operators_3d_channel_cylinder(Dproj, Gproj, Ap0, div_bc_unit, beta_p, alpha_u, alpha_v,
                                                 alpha_w, fluid_p, active_qu, active_qv, active_qw, id_p,
                                                 id_qu, id_qv, id_qw, par);
  SparseMatrix Au, Av, Aw, Ap;
  std::vector<double> scale_u, scale_v, scale_w;
  row_scale_sparse(Au0, Au, scale_u);
  row_scale_sparse(Av0, Av, scale_v);
  row_scale_sparse(Aw0, Aw, scale_w);
  Ap = Ap0;
  for (int i = 1; i <= Ap.nrows; ++i)
    for (auto &kv : Ap.rows[(size_t)(i - 1)]) kv.second = -kv.second;
  std::vector<int> fu, fv, fw, fp;
  build_flat_of_id_u(id_u, nx, ny, nz, fu);
  build_flat_of_id_v(id_v, nx, ny, nz, fv);
  build_flat_of_id_w(id_w, nx, ny, nz, fw);
  build_flat_of_id_p(id_p, nx, ny, nz, fp);
  std::vector<HYPRE_Complex> Au_vals, Av_vals, Aw_vals, Ap_vals;
  embed_u_matrix_to_rowmajor_3d(Au, fu, id_u, nx, ny, nz, Au_vals);
  embed_v_matrix_to_rowmajor_3d(Av, fv, id_v, nx, ny, nz, Av_vals);
  embed_w_matrix_to_rowmajor_3d(Aw, fw, id_w, nx, ny, nz, Aw_vals);
  embed_p_matrix_to_rowmajor_3d(Ap, fp, id_p, nx, ny, nz, Ap_vals);
  std::vector<double> uin;
  build_uin(uin, ny, nz, dy, dz, par.Ly, par.Um);

  rc->put("beta_p", beta_p); rc->put("alpha_u", alpha_u); rc->put("alpha_v", alpha_v); rc->put("alpha_w", alpha_w);
  rc->put("fluid_p", fluid_p); rc->put("active_u", active_u); rc->put("active_v", active_v);
  rc->put("active_w", active_w); rc->put("active_qu", active_qu); rc->put("active_qv", active_qv);
  rc->put("active_qw", active_qw);
  rc->put("id_u", id_u); rc->put("id_v", id_v); rc->put("id_w", id_w); rc->put("id_p", id_p);
  rc->put("id_qu", id_qu); rc->put("id_qv", id_qv); rc->put("id_qw", id_qw);
  rc->put("scale_u", scale_u); rc->put("scale_v", scale_v); rc->put("scale_w", scale_w);
  rc->put("rhs_u_bc", rhs_u_bc_unit); rc->put("rhs_v_bc", rhs_v_bc); rc->put("rhs_w_bc", rhs_w_bc);
  rc->put("div_bc_unit", div_bc_unit);
  rc->put("Au_vals", Au_vals); rc->put("Av_vals", Av_vals); rc->put("Aw_vals", Aw_vals); rc->put("Ap_vals", Ap_vals);
  rc->put("uin", uin);
  rc->put_csr("D", Dproj);
  rc->put_csr("G", Gproj);
  std::vector<int> counts = {(int)*std::max_element(id_u.begin(), id_u.end()),
                             (int)*std::max_element(id_v.begin(), id_v.end()),
                             (int)*std::max_element(id_w.begin(), id_w.end()),
                             (int)*std::max_element(id_p.begin(), id_p.end()),
                             (int)*std::max_element(id_qu.begin(), id_qu.end()),
                             (int)*std::max_element(id_qv.begin(), id_qv.end()),
                             (int)*std::max_element(id_qw.begin(), id_qw.end()), n_pruned};
  rc->put("counts", counts);
  return rc;
}

long ref_case_array_bytes(void *h, const char *name, int *elem) {
  RefCase *rc = (RefCase *)h;
  auto it = rc->arrays.find(name);
  if (it == rc->arrays.end()) return -1;
  if (elem) *elem = it->second.elem;
  return (long)it->second.bytes.size();
}

int ref_case_array_get(void *h, const char *name, void *dst, long nbytes) {
  RefCase *rc = (RefCase *)h;
  auto it = rc->arrays.find(name);
  if (it == rc->arrays.end() || (long)it->second.bytes.size() != nbytes) return -1;
  if (nbytes) std::memcpy(dst, it->second.bytes.data(), (size_t)nbytes);
  return 0;
}

void ref_case_free(void *h) { delete (RefCase *)h; }

// CPU twin of the BC cleanup (immersed_operators.hpp:1036-1053), in place.
void ref_enforce_bc(double *u, double *v, double *w, const unsigned char *au, const unsigned char *av,
                    const unsigned char *aw, const double *uin_step, int nx, int ny, int nz) {
  size_t NU = (size_t)(nx + 1) * ny * nz, NV = (size_t)nx * (ny + 1) * nz, NW = (size_t)nx * ny * (nz + 1);
  std::vector<double> U(u, u + NU), V(v, v + NV), W(w, w + NW), uin(uin_step, uin_step + (size_t)ny * nz);
  std::vector<char> AU(au, au + NU), AV(av, av + NV), AW(aw, aw + NW);
  enforce_bc_and_cleanup(U, V, W, AU, AV, AW, uin, nx, ny, nz);
  std::memcpy(u, U.data(), NU * 8); std::memcpy(v, V.data(), NV * 8); std::memcpy(w, W.data(), NW * 8);
}

// CPU twins of the centred convection (immersed_operators.hpp:990-1034).
void ref_convection(double *cu, double *cv, double *cw, const double *u, const double *v, const double *w,
                    const unsigned char *au, const unsigned char *av, const unsigned char *aw, int nx, int ny,
                    int nz, double dx, double dy, double dz) {
  size_t NU = (size_t)(nx + 1) * ny * nz, NV = (size_t)nx * (ny + 1) * nz, NW = (size_t)nx * ny * (nz + 1);
  std::vector<double> U(u, u + NU), V(v, v + NV), W(w, w + NW), CU, CV, CW, dummy;
  std::vector<char> AU(au, au + NU), AV(av, av + NV), AW(aw, aw + NW);
  compute_convective_u_centered_3d(CU, U, V, W, AU, dummy, nx, ny, nz, dx, dy, dz);
  compute_convective_v_centered_3d(CV, U, V, W, AV, nx, ny, nz, dx, dy, dz);
  compute_convective_w_centered_3d(CW, U, V, W, AW, nx, ny, nz, dx, dy, dz);
  std::memcpy(cu, CU.data(), NU * 8); std::memcpy(cv, CV.data(), NV * 8); std::memcpy(cw, CW.data(), NW * 8);
}

// The reference's VTK writer (immersed_operators.hpp:1055-1076) and its
// per-step file name (solver_helpers.hpp:470-482).
void ref_write_vtk(const char *path, const double *u, const double *v, const double *w, const double *p,
                   const unsigned char *fluid, int nx, int ny, int nz, double Lx, double Ly, double Lz) {
  size_t NU = (size_t)(nx + 1) * ny * nz, NV = (size_t)nx * (ny + 1) * nz, NW = (size_t)nx * ny * (nz + 1),
         NP = (size_t)nx * ny * nz;
  std::vector<double> U(u, u + NU), V(v, v + NV), W(w, w + NW), P(p, p + NP);
  std::vector<char> F(fluid, fluid + NP);
  write_vtk_cellcentered(path, U, V, W, P, F, nx, ny, nz, Lx, Ly, Lz);
}

int ref_vtk_step_name(const char *base, int step, char *out, int len) {
  const std::string s = vtk_filename_with_step(base, step);
  std::snprintf(out, (size_t)len, "%s", s.c_str());
  return (int)s.size();
}

}  // extern "C"
