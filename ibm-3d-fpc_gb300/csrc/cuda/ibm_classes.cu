// Record classes: the distinct records of an operator, kept once each.
//
// On a uniform Cartesian grid with immersed bodies almost every row of the
// momentum and pressure operators is the same: all fluid cells away from walls
// and bodies carry identical coefficients, and the rows that differ (cut
// cells, wall neighbours) repeat along the body and the walls. A 640 x 128 x
// 128 channel with a cylinder has 166 to 310 distinct rows per operator. A
// kernel that reads a 2-byte class per point and the record from a small table
// (resident in L1 / L2) moves 2 bytes instead of 28 to 112 per point, and
// computes with the same values bit for bit.
//
// Building: a 64-bit hash per record on the device, class numbers assigned on
// the host in first-seen order, the table gathered on the device, and every
// record compared bit for bit with its class's record (a hash collision makes
// the build fail, and the caller keeps the plain records).
#include <unordered_map>

#include "ibm_common.cuh"

namespace ibm {
namespace {

// splitmix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Hash of record t: its 32-bit words folded in order.
__global__ void k_hash_records(const unsigned *__restrict__ words, int wpr, long nrec,
                               unsigned long long *__restrict__ h) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nrec; t += (long)gridDim.x * blockDim.x) {
    const unsigned *w = words + t * wpr;
    unsigned long long z = 0x9e3779b97f4a7c15ull;
    for (int q = 0; q < wpr; ++q) z = mix64(z ^ ((unsigned long long)w[q] + ((unsigned long long)q << 32)));
    h[t] = z;
  }
}

__global__ void k_gather_classes(const unsigned *__restrict__ words, int wpr, const long *__restrict__ rep, int K,
                                 unsigned *__restrict__ tab) {
  const long total = (long)K * wpr;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long c = e / wpr;
    const int q = (int)(e - c * wpr);
    tab[e] = words[rep[c] * wpr + q];
  }
}

// Counts the records that differ from their class's record in any bit.
__global__ void k_verify_classes(const unsigned *__restrict__ words, int wpr, long nrec,
                                 const uint16_t *__restrict__ code, const unsigned *__restrict__ tab,
                                 unsigned *__restrict__ bad) {
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nrec; t += (long)gridDim.x * blockDim.x) {
    const unsigned *w = words + t * wpr;
    const unsigned *c = tab + (long)code[t] * wpr;
    bool same = true;
    for (int q = 0; q < wpr; ++q) same = same && w[q] == c[q];
    if (!same) atomicAdd(bad, 1u);
  }
}

int grid_of(long n) { return (int)std::max<long>(1, std::min<long>((n + kThreads - 1) / kThreads, 65535L * 8)); }

}  // namespace

template <class T>
bool build_classes(cudaStream_t st, const T *rec, int W, long nrec, Classes<T> &out) {
  static_assert(sizeof(T) % 4 == 0, "records are whole 32-bit words");
  out.code.release();
  out.tab.release();
  out.K = 0;
  out.W = W;
  if (nrec <= 0 || W <= 0) return false;
  const int wpr = (int)(W * sizeof(T) / 4);
  const unsigned *words = reinterpret_cast<const unsigned *>(rec);
  DBuf<unsigned long long> dh;
  dh.alloc((size_t)nrec);
  {
    LaunchScope ls(K_SETUP, st, 0.0);
    k_hash_records<<<grid_of(nrec), kThreads, 0, st>>>(words, wpr, nrec, dh.p);
  }
  std::vector<unsigned long long> h((size_t)nrec);
  IBM_CUDA_TRY(cudaMemcpyAsync(h.data(), dh.p, (size_t)nrec * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  dh.release();
  std::vector<uint16_t> code((size_t)nrec);
  std::vector<long> rep;
  std::unordered_map<unsigned long long, int> id;
  unsigned long long prev_h = 0;
  int prev_c = -1;
  for (long t = 0; t < nrec; ++t) {
    const unsigned long long v = h[(size_t)t];
    int c;
    if (prev_c >= 0 && v == prev_h) {
      c = prev_c;
    } else {
      auto it = id.find(v);
      if (it == id.end()) {
        if ((int)rep.size() >= kMaxClasses) return false;
        c = (int)rep.size();
        id.emplace(v, c);
        rep.push_back(t);
      } else {
        c = it->second;
      }
      prev_h = v;
      prev_c = c;
    }
    code[(size_t)t] = (uint16_t)c;
  }
  const int K = (int)rep.size();
  DBuf<long> drep;
  drep.alloc((size_t)K);
  DBuf<unsigned> bad;
  bad.alloc(1);
  out.code.alloc((size_t)nrec);
  out.tab.alloc((size_t)K * W);
  IBM_CUDA_TRY(cudaMemcpyAsync(drep.p, rep.data(), (size_t)K * sizeof(long), cudaMemcpyHostToDevice, st));
  IBM_CUDA_TRY(cudaMemcpyAsync(out.code.p, code.data(), (size_t)nrec * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
  bad.zero(st);
  {
    LaunchScope ls(K_SETUP, st, 0.0);
    k_gather_classes<<<grid_of((long)K * wpr), kThreads, 0, st>>>(words, wpr, drep.p, K,
                                                                   reinterpret_cast<unsigned *>(out.tab.p));
  }
  {
    LaunchScope ls(K_SETUP, st, 0.0);
    k_verify_classes<<<grid_of(nrec), kThreads, 0, st>>>(words, wpr, nrec, out.code.p,
                                                         reinterpret_cast<const unsigned *>(out.tab.p), bad.p);
  }
  unsigned nbad = 0;
  IBM_CUDA_TRY(cudaMemcpyAsync(&nbad, bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  IBM_CUDA_TRY(cudaStreamSynchronize(st));
  if (nbad != 0) {
    out.code.release();
    out.tab.release();
    return false;
  }
  out.K = K;
  return true;
}

template bool build_classes<float>(cudaStream_t, const float *, int, long, Classes<float> &);
template bool build_classes<double>(cudaStream_t, const double *, int, long, Classes<double> &);

}  // namespace ibm
