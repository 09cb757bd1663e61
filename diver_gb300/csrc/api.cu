// Library-level entry points: version and status names.
#include "common.cuh"

extern "C" {

int dv_version(void) { return 100; }

const char* dv_status_string(int status) {
  switch (status) {
    case DV_OK: return "ok";
    case DV_ERR_ARG: return "invalid argument";
    case DV_ERR_CUDA: return "CUDA error";
    case DV_ERR_OOM: return "out of device memory";
    case DV_ERR_TIMEOUT: return "bounded device wait timed out";
    case DV_ERR_OVERFLOW: return "capacity too small";
    case DV_ERR_UNSUPPORTED: return "unsupported device or option";
    default: return "unknown status";
  }
}

}  // extern "C"
