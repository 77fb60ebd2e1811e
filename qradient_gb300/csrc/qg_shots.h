// Per-term Pauli expectations and projector shots (qg_shots.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace qg {

constexpr int PAULI_BLOCKS = 1024;  // maximum grid of the expectation reduction
constexpr int PAULI_CHUNK = 64;     // terms per launch (passed by value)

struct PauliTerm {
  int8_t kind;  // QG_PAULI_X/Y/Z/ZZ
  int8_t b0;    // index bit of the (first) qubit: n - 1 - q0
  int8_t b1;    // ZZ: index bit of q1
  int8_t pad;
};

struct PauliChunk {
  int count;
  PauliTerm term[PAULI_CHUNK];
};

size_t pauli_workspace_bytes(int nterms);

template <typename C>
cudaError_t launch_pauli_expectations(int n, const C* psi, int nterms, const PauliTerm* terms, double* ws,
                                      double* out, cudaStream_t st);

}  // namespace qg
