// Allocation-free RI-J response, for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside another
// framework's memory pool or allocator hooks, work recorded into a CUDA graph by a host
// that forbids allocation during capture, or embedded runtimes with a fixed device-memory
// budget.  cphf_rij_response_bra_noalloc gives them the Coulomb part of the RI-JK
// response without any allocation: the caller passes every input and the output as device
// pointers, and the one intermediate (the aux-space density d[naux, nb]) lives in the
// file-scope array below.  That array is part of the library image: every GPU that loads
// libcphf holds its 8 MiB until the process exits.
#include <mutex>

#include "../../include/cphf.h"
#include "gemm_simt.cuh"

namespace {

constexpr int64_t kScratchElems = int64_t(1) << 20;  // FP64 elements: naux * nb must not exceed this
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_rij_scratch[kScratchElems];

// Device address of g_rij_scratch, resolved once per device with that device current.
double* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

}  // namespace

extern "C" int64_t cphf_rij_noalloc_capacity(void) { return kScratchElems; }

extern "C" cphf_status cphf_rij_response_bra_noalloc(const double* Z, const double* bra, int64_t nao,
                                                     int64_t nocc, int64_t naux, int64_t nb, double scale_j,
                                                     double* out, void* stream) {
  if (!Z || !bra || !out || nao <= 0 || nocc <= 0 || naux <= 0 || nb < 0) return CPHF_ERR_ARG;
  if (nb > kScratchElems / naux) return CPHF_ERR_ARG;  // naux * nb beyond the static scratch (no overflow)
  if (nb == 0) return CPHF_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return CPHF_ERR_CUDA;
  }
  double* d = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      // The host-side symbol is only a stand-in: the kernels need the device address.
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_rij_scratch) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return CPHF_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<double*>(p);
    }
    d = g_scratch_addr[dev];
  }
  int sms = 152;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sms = 152;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // d[P, a] = 2 sum_(mu,i) Z[mu, i, P] bra[mu, i, a]   (d_P = sum B_P (D1 + D1^T), src/ri_jk/hess_r.rs:131-137)
  // Every element of d is written (beta = 0): nothing left from an earlier call is read.
  cphf::GemmDesc g1;
  g1.M = naux; g1.N = nb; g1.K = nao * nocc;
  g1.A = Z; g1.a_m = nao * nocc; g1.a_k = 1;
  g1.B = bra; g1.b_k = 1; g1.b_n = nao * nocc;
  g1.C = d; g1.c_m = 1; g1.c_n = naux;
  g1.alpha = 2.0; g1.beta = 0.0;
  // out[(mu,i), a] = scale_j * 2 sum_P Z[(mu,i), P] d[P, a]   (J Cocc, hess_r.rs:138-139, 1946)
  cphf::GemmDesc g2;
  g2.M = nao * nocc; g2.N = nb; g2.K = naux;
  g2.A = Z; g2.a_m = 1; g2.a_k = nao * nocc;
  g2.B = d; g2.b_k = 1; g2.b_n = naux;
  g2.C = out; g2.c_m = 1; g2.c_n = nao * nocc;
  g2.alpha = 2.0 * scale_j; g2.beta = 0.0;
  // no workspace: the GEMMs run without split-K and allocate nothing
  if (cphf::gemm<double, double, double, double>(g1, s, nullptr, 0, sms) != cudaSuccess) return CPHF_ERR_CUDA;
  if (cphf::gemm<double, double, double, double>(g2, s, nullptr, 0, sms) != cudaSuccess) return CPHF_ERR_CUDA;
  return CPHF_OK;
}
