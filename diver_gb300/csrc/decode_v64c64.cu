// DIVeR decoder variant: width 64, 64-channel features (plain FP32).
#include "decode.cuh"

namespace dv {

int decode_fwd_v64c64(const DecodeArgs& a, cudaStream_t st, int sms) {
  return launch_decode_fwd<64, 64, 1, 128>(a, st, sms);
}

int decode_bwd_v64c64(const DecodeArgs& a, cudaStream_t st, int sms) {
  return launch_decode_bwd<64, 64, 1, 64>(a, st, sms);
}

}  // namespace dv
