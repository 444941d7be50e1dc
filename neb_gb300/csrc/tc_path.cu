// Tensor-core (tcgen05) path: placeholder entry points until the sm_103a
// kernels land; they report NEB_ERR_UNSUPPORTED.
#include "tc_path.cuh"

namespace neb {

size_t tc_workspace_bytes(const neb_net*, int64_t) { return 0; }

int tc_forward(const neb_net*, const float* const*, const float* const*, const float*, int64_t,
               const TcTape&, char*, cudaStream_t) {
  set_error("NEB_PREC_BF16X3 forward not built");
  return NEB_ERR_UNSUPPORTED;
}
int tc_output(const neb_net*, const float*, const float*, int, int, int64_t, const void*, void*,
              cudaStream_t) {
  set_error("NEB_PREC_BF16X3 output not built");
  return NEB_ERR_UNSUPPORTED;
}
int tc_hidden_gram(const neb_net*, const float*, int64_t, const void*, double*, double*, char*,
                   char*, cudaStream_t) {
  set_error("NEB_PREC_BF16X3 hidden gram not built");
  return NEB_ERR_UNSUPPORTED;
}
int tc_backward_hidden(const neb_net*, const float* const*, const double*, const double*,
                       const float*, int64_t, const TcTape&, float* const*, float* const*, char*,
                       size_t, char*, char*, char*, cudaStream_t) {
  set_error("NEB_PREC_BF16X3 backward not built");
  return NEB_ERR_UNSUPPORTED;
}

}  // namespace neb
