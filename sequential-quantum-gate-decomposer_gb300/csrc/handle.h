// Definition of the opaque circuit handle shared by the engine's translation units, and
// the thread-local error text behind sqg_last_error().
#pragma once
#include <string>
#include <vector>

#include "gates.cuh"

struct sqg_circuit {
  int n = 0, N = 0, L = 0, P = 0;
  int device = 0;
  sqg::Gate* d_gates = nullptr;
  std::vector<sqg::Gate> h_gates;
};

namespace sqg {
// Records msg as the calling thread's last error and returns status.
int set_error(int status, const std::string& msg);
}  // namespace sqg
