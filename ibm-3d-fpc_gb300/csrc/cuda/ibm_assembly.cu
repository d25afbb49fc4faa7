// GPU assembly of the momentum and pressure operators (ibm_assemble_momentum,
// ibm_assemble_pressure): one thread per row, the row arithmetic of
// ibm_assembly.cuh.
#include <algorithm>

#include "ibm_assembly.cuh"
#include "ibm_common.cuh"

namespace ibm {

namespace {

// rows[r][7] and scale[id] (index 0 untouched) of field f's solve box.
__global__ void k_assemble_momentum(int f, long n, asmb::Geo g, const unsigned char *act, const int *id,
                                    double *rows, double *scale) {
  for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    double a[7];
    int P = 0;
    const double sc = asmb::momentum_row(f, r, g, act, id, a, &P);
    for (int t = 0; t < 7; ++t) rows[7 * r + t] = a[t];
    if (P > 0) scale[P] = sc;
  }
}

__global__ void k_assemble_pressure(long n, asmb::Geo g, asmb::PInputs in, double *rows) {
  for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x)
    asmb::pressure_row(c, g, in, rows + 7 * c);
}

}  // namespace

void launch_assemble_pressure(cudaStream_t st, long n, const asmb::Geo &g, const asmb::PInputs &in, double *rows) {
  LaunchScope ls(K_SETUP, st, 120.0 * n);
  const long b = std::max(1L, std::min((n + kThreads - 1) / kThreads, (long)sm_count() * 8));
  k_assemble_pressure<<<(int)b, kThreads, 0, st>>>(n, g, in, rows);
}

void launch_assemble_momentum(cudaStream_t st, int f, long n, const asmb::Geo &g, const unsigned char *act,
                              const int *id, double *rows, double *scale) {
  LaunchScope ls(K_SETUP, st, 64.0 * n);
  const long b = std::max(1L, std::min((n + kThreads - 1) / kThreads, (long)sm_count() * 8));
  k_assemble_momentum<<<(int)b, kThreads, 0, st>>>(f, n, g, act, id, rows, scale);
}

}  // namespace ibm
