// Host check of the GPU assembly's row arithmetic (ibm_assembly.cuh, built
// for the host with unfused IEEE operations) against the CPU setup
// (libibmhost): every row value and row scale of the three momentum
// operators and every row of the pressure operator, bit for bit. Usage: assembly_check nx ny nz [Um Rcirc ycirc nu dt]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>

#include "ibm_host.h"
#include "../ibm-3d-fpc_gb300/csrc/cuda/ibm_assembly.cuh"

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  ibm_case_params p;
  ibm_case_params_default(&p);
  p.nx = atoi(argv[1]); p.ny = atoi(argv[2]); p.nz = atoi(argv[3]);
  p.Lx = 2.5; p.Ly = 0.41; p.Lz = 0.41; p.xcirc = 0.5; p.ycirc = 0.2; p.Rcirc = 0.05;
  if (argc > 4) p.Um = atof(argv[4]);
  if (argc > 5) p.Rcirc = atof(argv[5]);
  if (argc > 6) p.ycirc = atof(argv[6]);
  if (argc > 7) p.nu = atof(argv[7]);
  if (argc > 8) p.dt = atof(argv[8]);
  ibm_case *c = nullptr;
  if (ibm_case_build(&p, &c) != 0) return 3;
  ibm::asmb::Geo g{p.nx, p.ny, p.nz, p.Lx, p.Ly, p.Lz, p.rho, p.nu, p.dt, p.xcirc, p.ycirc, p.Rcirc};
  const char *act[3] = {"active_u", "active_v", "active_w"}, *ids[3] = {"id_u", "id_v", "id_w"};
  const char *vals[3] = {"Au_vals", "Av_vals", "Aw_vals"}, *scs[3] = {"scale_u", "scale_v", "scale_w"};
  const long nb[3] = {(long)(p.nx - 1) * p.ny * p.nz, (long)p.nx * (p.ny - 1) * p.nz, (long)p.nx * p.ny * (p.nz - 1)};
  long bad = 0, rows = 0;
  for (int f = 0; f < 3; ++f) {
    const unsigned char *a = (const unsigned char *)ibm_case_array(c, act[f]);
    const int *id = (const int *)ibm_case_array(c, ids[f]);
    const double *ref = (const double *)ibm_case_array(c, vals[f]);
    const double *rsc = (const double *)ibm_case_array(c, scs[f]);
    for (long r = 0; r < nb[f]; ++r) {
      double row[7];
      int P = 0;
      const double sc = ibm::asmb::momentum_row(f, r, g, a, id, row, &P);
      ++rows;
      bool ok = std::memcmp(row, ref + 7 * r, sizeof(row)) == 0;
      if (P > 0) ok = ok && std::memcmp(&sc, rsc + P, sizeof(double)) == 0;
      if (!ok && bad < 5) std::printf("field %d row %ld differs\n", f, r);
      bad += ok ? 0 : 1;
    }
  }
  // pressure rows
  ibm::asmb::PInputs in;
  in.fluid = (const unsigned char *)ibm_case_array(c, "fluid_p");
  in.id_p = (const int *)ibm_case_array(c, "id_p");
  in.beta = (const double *)ibm_case_array(c, "beta_p");
  const char *al[3] = {"alpha_u", "alpha_v", "alpha_w"}, *aq[3] = {"active_qu", "active_qv", "active_qw"},
             *iq[3] = {"id_qu", "id_qv", "id_qw"};
  for (int f = 0; f < 3; ++f) {
    in.alpha[f] = (const double *)ibm_case_array(c, al[f]);
    in.act_q[f] = (const unsigned char *)ibm_case_array(c, aq[f]);
    in.id_q[f] = (const int *)ibm_case_array(c, iq[f]);
  }
  ibm_case_counts cnt;
  ibm_case_get_counts(c, &cnt);
  in.nQu = cnt.nqu; in.nQv = cnt.nqv;
  const double *ap = (const double *)ibm_case_array(c, "Ap_vals");
  const long np = (long)p.nx * p.ny * p.nz;
  for (long cell = 0; cell < np; ++cell) {
    double row[7];
    ibm::asmb::pressure_row(cell, g, in, row);
    ++rows;
    const bool ok = std::memcmp(row, ap + 7 * cell, sizeof(row)) == 0;
    if (!ok && bad < 5) std::printf("pressure cell %ld differs\n", cell);
    bad += ok ? 0 : 1;
  }
  std::printf("rows %ld mismatches %ld\n", rows, bad);
  ibm_case_free(c);
  return bad == 0 ? 0 : 1;
}
