// DIVeR decoder variant: width 32, 32-channel features (plain FP32).
#include "decode.cuh"

namespace dv {

int decode_fwd_v32c32(const DecodeArgs& a, cudaStream_t st, int sms) {
  return launch_decode_fwd<32, 32, 2, 128>(a, st, sms);
}

int decode_bwd_v32c32(const DecodeArgs& a, cudaStream_t st, int sms) {
  return launch_decode_bwd<32, 32, 2, 128>(a, st, sms);
}

}  // namespace dv
