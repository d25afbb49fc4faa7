// ibm_run — the reference's application (main.cu) on the GB300 solver.
//
// Accepts the reference's flags (common.hpp:87-127) plus a few for the
// solver options this implementation adds, builds the case on the CPU with
// libibmhost (bit-identical to the reference's setup), hands it to the C ABI
// of libibmgpu and prints the reference's per-step table (main.cu:244,
// 365-368) and timing summary (main.cu:380-389).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ibm_gpu.h"
#include "ibm_host.h"

namespace {

struct Options {
  ibm_case_params cp;
  int nsteps = 10, print_every = 1, inlet_ramp_steps = 200, device = 0;
  ibm_solver_params sp;
  int checkpoint_every = 0;
  std::string checkpoint_prefix = "ibm_state";
  std::string restart;      // checkpoint file to resume from (its step + 1 is the first step run)
  std::string case_cache;   // case cache file (ibm_case_build_cached)
  // VTK output with the reference's flags and file names (common.hpp:82-84,
  // main.cu:370-378); off unless -write-vtk 1 is given: the reference's
  // default writes an ASCII file every step, outside the hot path
  int write_vtk = 0, vtk_every = 0;
  std::string vtk_filename = "st3d_channel_cylinder_struct_mac_cuda.vtk";
};

bool arg(int &a, int argc, char **argv, const char *name) { return !std::strcmp(argv[a], name) && a + 1 < argc; }

void parse(int argc, char **argv, Options &o) {
  for (int a = 1; a < argc; ++a) {
    if (arg(a, argc, argv, "-nx")) o.cp.nx = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-ny")) o.cp.ny = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-nz")) o.cp.nz = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-Lx")) o.cp.Lx = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-Ly")) o.cp.Ly = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-Lz")) o.cp.Lz = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-rho")) o.cp.rho = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-nu")) o.cp.nu = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-Um")) o.cp.Um = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-dt")) o.cp.dt = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-nsteps")) o.nsteps = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-print-every")) o.print_every = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-inlet-ramp-steps")) o.inlet_ramp_steps = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-use-zero-initial-guess")) o.sp.use_zero_initial_guess = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-device")) o.device = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-nsub-beta")) o.cp.nsub_beta = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-beta-tol")) o.cp.beta_tol = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-alpha-tol")) o.cp.alpha_tol = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-xcirc")) o.cp.xcirc = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-ycirc")) o.cp.ycirc = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-Rcirc")) o.cp.Rcirc = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-vel-maxit")) o.sp.vel_maxit = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-vel-kdim")) o.sp.vel_kdim = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-vel-tol")) o.sp.vel_tol = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-vel-print")) ++a;  // printing of solver internals: not reproduced
    else if (arg(a, argc, argv, "-vel-jacobi-iters")) o.sp.vel_jacobi_iters = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-p-maxit")) o.sp.p_maxit = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-p-kdim")) o.sp.p_kdim = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-p-tol")) o.sp.p_tol = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-p-print")) ++a;
    else if (arg(a, argc, argv, "-p-pc-maxit")) o.sp.p_pc_maxit = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-p-pc-relax-type")) o.sp.p_pc_relax_type = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-p-pc-rap-type")) o.sp.p_pc_rap_type = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-write-vtk")) o.write_vtk = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-vtk-every")) o.vtk_every = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-vtk")) o.vtk_filename = argv[++a];
    // options of this implementation
    else if (arg(a, argc, argv, "-precision")) o.sp.precision = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-use-graph")) o.sp.use_graph = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-mg-group-ratio")) o.sp.mg_group_ratio = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-mg-omega")) o.sp.mg_omega = std::atof(argv[++a]);
    else if (arg(a, argc, argv, "-vel-inner-sweeps")) o.sp.vel_inner_sweeps = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-checkpoint-every")) o.checkpoint_every = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-checkpoint")) o.checkpoint_prefix = argv[++a];
    else if (arg(a, argc, argv, "-restart")) o.restart = argv[++a];
    else if (arg(a, argc, argv, "-forces")) o.sp.compute_forces = std::atoi(argv[++a]);
    else if (arg(a, argc, argv, "-case-cache")) o.case_cache = argv[++a];
  }
}

template <class T>
const T *arr(const ibm_case *c, const char *name) {
  return static_cast<const T *>(ibm_case_array(c, name));
}

int fail(const char *what, ibm_ctx *ctx) {
  std::fprintf(stderr, "%s: %s\n", what, ibm_last_error(ctx));
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  ibm_case_params_default(&o.cp);
  ibm_solver_params_default(&o.sp);
  parse(argc, argv, o);
  char dev[256] = "";
  if (ibm_device_query(o.device, dev, sizeof(dev)) == IBM_OK) std::printf("GPU                   : %s\n", dev);

  const auto t_setup0 = std::chrono::steady_clock::now();
  ibm_case *cs = nullptr;
  if (o.case_cache.empty() ? ibm_case_build(&o.cp, &cs) != 0
                           : ibm_case_build_cached(&o.cp, o.case_cache.c_str(), &cs) != 0) {
    std::fprintf(stderr, "case setup failed (bad parameters)\n");
    return 1;
  }
  ibm_case_counts cnt;
  ibm_case_get_counts(cs, &cnt);
  const int nx = o.cp.nx, ny = o.cp.ny, nz = o.cp.nz;
  ibm_grid_desc g{nx, ny, nz, o.cp.Lx, o.cp.Ly, o.cp.Lz, o.cp.rho, o.cp.nu, o.cp.dt, o.device};
  ibm_ctx *ctx = nullptr;
  if (ibm_create(&g, &ctx) != IBM_OK) return fail("ibm_create", nullptr);
  if (ibm_set_operator(ctx, IBM_FIELD_U, arr<double>(cs, "Au_vals"), nx - 1, ny, nz) ||
      ibm_set_operator(ctx, IBM_FIELD_V, arr<double>(cs, "Av_vals"), nx, ny - 1, nz) ||
      ibm_set_operator(ctx, IBM_FIELD_W, arr<double>(cs, "Aw_vals"), nx, ny, nz - 1) ||
      ibm_set_operator(ctx, IBM_FIELD_P, arr<double>(cs, "Ap_vals"), nx, ny, nz))
    return fail("ibm_set_operator", ctx);
  if (ibm_set_masks(ctx, arr<uint8_t>(cs, "active_u"), arr<uint8_t>(cs, "active_v"), arr<uint8_t>(cs, "active_w"),
                    arr<uint8_t>(cs, "fluid_p"), arr<uint8_t>(cs, "active_qu"), arr<uint8_t>(cs, "active_qv"),
                    arr<uint8_t>(cs, "active_qw"), arr<int32_t>(cs, "id_u"), arr<int32_t>(cs, "id_v"),
                    arr<int32_t>(cs, "id_w"), arr<int32_t>(cs, "id_p"), arr<int32_t>(cs, "id_qu"),
                    arr<int32_t>(cs, "id_qv"), arr<int32_t>(cs, "id_qw")))
    return fail("ibm_set_masks", ctx);
  if (ibm_set_aux(ctx, arr<double>(cs, "scale_u"), arr<double>(cs, "scale_v"), arr<double>(cs, "scale_w"),
                  arr<double>(cs, "rhs_u_bc"), arr<double>(cs, "rhs_v_bc"), arr<double>(cs, "rhs_w_bc"),
                  arr<double>(cs, "div_bc_unit"), arr<double>(cs, "uin")))
    return fail("ibm_set_aux", ctx);
  if (ibm_set_projection_csr(ctx, arr<int32_t>(cs, "D_rowptr"), arr<int32_t>(cs, "D_col"), arr<double>(cs, "D_val"),
                             cnt.np, arr<int32_t>(cs, "G_rowptr"), arr<int32_t>(cs, "G_col"),
                             arr<double>(cs, "G_val"), cnt.nqu + cnt.nqv + cnt.nqw))
    return fail("ibm_set_projection_csr", ctx);
  if (ibm_set_solver_params(ctx, &o.sp)) return fail("ibm_set_solver_params", ctx);
  // initial state (main.cu:116-126): zero fields, then the BC cleanup with the
  // unramped inlet profile
  std::vector<double> u((size_t)(nx + 1) * ny * nz, 0.0), v((size_t)nx * (ny + 1) * nz, 0.0),
      w((size_t)nx * ny * (nz + 1), 0.0), p((size_t)nx * ny * nz, 0.0);
  const double *uin = arr<double>(cs, "uin");
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j) u[((size_t)k * ny + j) * (nx + 1)] = uin[(size_t)j + (size_t)ny * k];
  int first_step = 1;
  if (!o.restart.empty()) {
    // checkpoint layout: int nx, ny, nz, step; double ramp; u, v, w, p
    std::FILE *f = std::fopen(o.restart.c_str(), "rb");
    int hdr[4] = {0, 0, 0, 0};
    double ramp0 = 0.0;
    bool ok = f && std::fread(hdr, sizeof(int), 4, f) == 4 && std::fread(&ramp0, sizeof(double), 1, f) == 1 &&
              hdr[0] == nx && hdr[1] == ny && hdr[2] == nz && hdr[3] >= 0 &&
              std::fread(u.data(), sizeof(double), u.size(), f) == u.size() &&
              std::fread(v.data(), sizeof(double), v.size(), f) == v.size() &&
              std::fread(w.data(), sizeof(double), w.size(), f) == w.size() &&
              std::fread(p.data(), sizeof(double), p.size(), f) == p.size();
    if (f) std::fclose(f);
    if (!ok) {
      std::fprintf(stderr, "restart: %s is not a checkpoint of a %d x %d x %d grid\n", o.restart.c_str(), nx, ny, nz);
      return 1;
    }
    first_step = hdr[3] + 1;
  }
  if (ibm_set_fields(ctx, u.data(), v.data(), w.data(), p.data())) return fail("ibm_set_fields", ctx);
  const double setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_setup0).count();

  std::printf("============================================================\n");
  std::printf("3D Schaefer-Turek channel with immersed full-height cylinder (GB300 solver)\n");
  std::printf("Grid                  : %d x %d x %d pressure cells\n", nx, ny, nz);
  std::printf("Domain                : [0,%g] x [0,%g] x [0,%g]\n", o.cp.Lx, o.cp.Ly, o.cp.Lz);
  std::printf("Cylinder center/rad   : (%.6f, %.6f), %.6f\n", o.cp.xcirc, o.cp.ycirc, o.cp.Rcirc);
  std::printf("nu                    : %.6e\n", o.cp.nu);
  std::printf("dt                    : %.6e\n", o.cp.dt);
  std::printf("nsteps                : %d\n", o.nsteps);
  std::printf("Pressure cells        : %d\n", cnt.np);
  std::printf("Active u/v/w          : %d / %d / %d\n", cnt.nu, cnt.nv, cnt.nw);
  std::printf("Projection q faces    : %d / %d / %d\n", cnt.nqu, cnt.nqv, cnt.nqw);
  std::printf("Pruned isolated x-y columns: %d\n", cnt.n_pruned);
  std::printf("Precision             : %s%s\n", o.sp.precision ? "FP32 preconditioners in FP64 flexible GMRES" : "FP64",
              o.sp.use_graph ? ", graph-captured step" : "");
  std::printf("Setup                 : %.3f s\n", setup_s);
  std::printf("============================================================\n");
  std::printf("step  ramp         max|u|         max|v|         max|w|         divL2          its(u,v,w,p)                relres(u,v,w,p)\n");
  double t_rhs = 0, t_mom = 0, t_p = 0, t_total = 0;
  const auto t0 = std::chrono::steady_clock::now();
  int rc_final = 0;
  for (int step = first_step; step <= o.nsteps; ++step) {
    const double ramp = std::min(1.0, (double)step / (double)o.inlet_ramp_steps);
    ibm_step_stats st;
    const int rc = ibm_step(ctx, ramp, &st);
    if (rc < 0) {
      std::fprintf(stderr, "step %d: %s\n", step, ibm_last_error(ctx));
      rc_final = 1;
      break;
    }
    t_rhs += st.t_rhs_ms; t_mom += st.t_mom_ms; t_p += st.t_p_ms; t_total += st.t_total_ms;
    if (step == 1 || step == o.nsteps || (o.print_every > 0 && step % o.print_every == 0)) {
      std::printf("%4d  %.6f  %.6e  %.6e  %.6e  %.6e  (%d,%d,%d,%d)  (%.3e,%.3e,%.3e,%.3e)", step, ramp, st.umax,
                  st.vmax, st.wmax, st.div_l2, st.u.iters, st.v.iters, st.w.iters, st.p.iters, st.u.rel_res,
                  st.v.rel_res, st.w.rel_res, st.p.rel_res);
      if (o.sp.compute_forces) {
        // drag / lift coefficients of the benchmark channel: 2 F / (rho U^2 D H), U = 4 Um / 9
        const double um = 4.0 * o.cp.Um / 9.0, sc = 2.0 / (o.cp.rho * um * um * 2.0 * o.cp.Rcirc * o.cp.Lz);
        std::printf("  cD %.5f cL %.5f", st.force[0] * sc, st.force[1] * sc);
      }
      std::printf("\n");
    }
    if (o.write_vtk && (step == 1 || step == o.nsteps || step % std::max(1, o.vtk_every) == 0)) {
      ibm_get_fields(ctx, u.data(), v.data(), w.data(), p.data());
      char name[4096];
      ibm_vtk_step_name(o.vtk_filename.c_str(), step, name, (int)sizeof(name));
      if (ibm_write_vtk(name, u.data(), v.data(), w.data(), p.data(), arr<uint8_t>(cs, "fluid_p"), nx, ny, nz,
                        o.cp.Lx, o.cp.Ly, o.cp.Lz) != 0)
        std::fprintf(stderr, "step %d: could not write %s\n", step, name);
    }
    if (o.checkpoint_every > 0 && step % o.checkpoint_every == 0) {
      ibm_get_fields(ctx, u.data(), v.data(), w.data(), p.data());
      const std::string fn = o.checkpoint_prefix + "_" + std::to_string(step) + ".bin";
      if (std::FILE *f = std::fopen(fn.c_str(), "wb")) {
        const int hdr[4] = {nx, ny, nz, step};
        std::fwrite(hdr, sizeof(int), 4, f);
        std::fwrite(&ramp, sizeof(double), 1, f);
        std::fwrite(u.data(), sizeof(double), u.size(), f);
        std::fwrite(v.data(), sizeof(double), v.size(), f);
        std::fwrite(w.data(), sizeof(double), w.size(), f);
        std::fwrite(p.data(), sizeof(double), p.size(), f);
        std::fclose(f);
      }
    }
  }
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("============================================================\n");
  std::printf("Timing summary\n");
  std::printf("momentum build time    : %.6e s\n", t_rhs * 1e-3);
  std::printf("momentum solve time    : %.6e s\n", t_mom * 1e-3);
  std::printf("pressure solve time    : %.6e s\n", t_p * 1e-3);
  std::printf("total wall time        : %.6e s\n", wall);
  std::printf("steps/s                : %.3f\n", (o.nsteps - first_step + 1) / std::max(wall, 1e-12));
  std::printf("kernel launches        : %lld\n", ibm_kernel_launches(ctx));
  std::printf("============================================================\n");
  ibm_destroy(ctx);
  ibm_case_free(cs);
  return rc_final;
}
