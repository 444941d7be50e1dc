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
// Tape layout of the tensor-core path (offsets of X_l and Z_l); returns total bytes.
size_t tc_tape_bytes(const neb_net* net, int64_t n, size_t* x_off, size_t* z_off);
// Synchronises the stream and reads the bounded-wait status word (0 = ok).
int tc_read_status(const neb_net* net, int64_t n, char* ws, cudaStream_t s, int* out);
// Runs the bounded-wait self-test kernel, synchronises and returns its status word.
int tc_wait_selftest(int arrive, uint32_t limit, int* status, cudaStream_t s, int* out);
int tc_forward(const neb_net* net, const float* const* W, const float* const* b, const float* feats,
               int64_t n, const TcTape& tape, char* ws, cudaStream_t s);
int tc_output(const neb_net* net, const float* Wout, const float* bout, int start, int stop,
              int64_t n, const void* tape, void* psi, cudaStream_t s);
int tc_hidden_gram(const neb_net* net, const float* qw, int64_t n, const void* hl, double* AM,
                   double* AS, int accumulate, char* ws, cudaStream_t s);
int tc_backward_hidden(const neb_net* net, const double* GMh, const double* GSh, const float* qw,
                       int64_t n, const TcTape& tape, float* const* gW, float* const* gb,
                       int accumulate, char* ws, cudaStream_t s);

}  // namespace neb
