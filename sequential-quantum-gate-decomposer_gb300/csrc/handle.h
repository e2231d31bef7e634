// Definition of the opaque circuit handle shared by the engine's translation units, and
// the thread-local error text behind sqg_last_error().
#pragma once
#include <string>
#include <vector>

#include "gates.cuh"

// Fused state-vector passes (sqg_apply_state): consecutive gates whose qubits, together with
// the lowest ones, fit one chunk of 2^K amplitudes form a block applied in shared memory.
struct sqg_state_block {
  int g0, g1;  // gates [g0, g1)
};

struct sqg_circuit {
  int n = 0, N = 0, L = 0, P = 0;
  int device = 0;
  sqg::Gate* d_gates = nullptr;
  std::vector<sqg::Gate> h_gates;
  // state-vector plan: chunk qubits K, blocks, gate records with chunk-local qubit positions,
  // per block the global offsets of the chunk's high local bits (2^(K - low) ints, padded to
  // 128) and the qubits that number the chunks (padded to 32)
  int sK = 0;
  std::vector<sqg_state_block> sblocks;
  sqg::Gate* d_lgates = nullptr;
  int* d_hitab = nullptr;
  int* d_inact = nullptr;
  // merged forward plan (Lm > 0 when it saves work): runs of single-qubit gates on one qubit
  // with no two-qubit gate on that qubit between them become one general 2x2 gate; d_mgates
  // holds the Lm records, members d_mmembers[d_mfirst[m] .. d_mfirst[m + 1]) their source gates
  int Lm = 0;
  sqg::Gate* d_mgates = nullptr;
  int* d_mfirst = nullptr;
  int* d_mmembers = nullptr;
};

namespace sqg {
// Records msg as the calling thread's last error and returns status.
int set_error(int status, const std::string& msg);
// Environment-matrix cost and gradient for qbit_num <= 5 (decompose.cu); SQG_ERR_UNSUPPORTED
// for shapes it does not take.
int env_cost_grad(const sqg_circuit* c, const double* theta, int B, const void* target, int cols, long long tstride,
                  int off, int variant, double* cost, double* grad, void* stream);
}  // namespace sqg
