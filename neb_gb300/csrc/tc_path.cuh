// Tensor-core (tcgen05, split-BF16) path of the jet MLP: declarations shared
// with the C-ABI dispatcher.
#pragma once
#include "neb_common.cuh"

namespace neb {

struct TcTape {
  void* x[NEB_MAX_HIDDEN + 1];  // layer inputs: hi plane then lo plane (bf16)
  void* z[NEB_MAX_HIDDEN + 1];  // pre-activations (float)
};

size_t tc_workspace_bytes(const neb_net* net, int64_t n);
int tc_forward(const neb_net* net, const float* const* W, const float* const* b, const float* feats,
               int64_t n, const TcTape& tape, char* ws, cudaStream_t s);
int tc_output(const neb_net* net, const float* Wout, const float* bout, int start, int stop,
              int64_t n, const void* tape, void* psi, cudaStream_t s);
int tc_hidden_gram(const neb_net* net, const float* qw, int64_t n, const void* hl, double* AM,
                   double* AS, char* part, char* ws, cudaStream_t s);
int tc_backward_hidden(const neb_net* net, const float* const* W, const double* GMh,
                       const double* GSh, const float* qw, int64_t n, const TcTape& tape,
                       float* const* gW, float* const* gb, char* zbuf, size_t zb1_off, char* part,
                       char* partb, char* ws, cudaStream_t s);

}  // namespace neb
