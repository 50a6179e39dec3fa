// D3Q27 instantiations of the fused sweep (see sweep.cuh).
#include "sweep.cuh"

namespace cflbm {

cudaError_t launch_sweep_q27(int store, int compute, const SweepArgs &a, cudaStream_t s) {
  // Double-float sweep: 5 blocks per SM (96 registers; measured at 512x128x128:
  // 3 / 4 / 5 per SM give 3,961 / 3,955 / 4,154 M cell updates/s).
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_sweep_t<27, double, df64, 5>(a, s) : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_sweep_t<27, double, double, 3>(a, s);
      case STORE_F32: return launch_sweep_t<27, float, double, 3>(a, s);
      case STORE_F16: return launch_sweep_t<27, F16Dev, double, 3>(a, s);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_sweep_t<27, double, float, 4>(a, s);
      case STORE_F32: return launch_sweep_t<27, float, float, 4>(a, s);
      case STORE_F16: return launch_sweep_t<27, F16Dev, float, 4>(a, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_channel_q27(int store, int compute, const SweepArgs &a,
                                      cudaStream_t s, const SweepFork *fk) {
  // Double-float channel sweep: 5 blocks per SM (102 registers; 3 / 4 / 5 / 6
  // per SM give 6,839 / 6,972 / 7,468 / 7,434 M cell updates/s at 512x128x128).
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_sweep_channel_t<27, double, df64, 5, 2>(a, s, fk)
                              : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_sweep_channel_t<27, double, double, 3, 2>(a, s, fk);
      case STORE_F32: return launch_sweep_channel_t<27, float, double, 3, 2>(a, s, fk);
      case STORE_F16: return launch_sweep_channel_t<27, F16Dev, double, 3, 2>(a, s, fk);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_sweep_channel_t<27, double, float, 8, 4>(a, s, fk);
      case STORE_F32: return launch_sweep_channel_t<27, float, float, 8, 4>(a, s, fk);
      case STORE_F16: return launch_sweep_channel_t<27, F16Dev, float, 8, 4>(a, s, fk);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_macros_channel_q27(int store, int compute, const SweepArgs &a,
                                      cudaStream_t s) {
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_macros_channel_t<27, double, df64>(a, s)
                              : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_macros_channel_t<27, double, double>(a, s);
      case STORE_F32: return launch_macros_channel_t<27, float, double>(a, s);
      case STORE_F16: return launch_macros_channel_t<27, F16Dev, double>(a, s);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_macros_channel_t<27, double, float>(a, s);
      case STORE_F32: return launch_macros_channel_t<27, float, float>(a, s);
      case STORE_F16: return launch_macros_channel_t<27, F16Dev, float>(a, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_stream_state_q27(int store, const SweepArgs &a, bool ref, double *out,
                                    cudaStream_t s) {
  switch (store) {
    case STORE_F64: return launch_stream_state_t<27, double>(a, ref, out, s);
    case STORE_F32: return launch_stream_state_t<27, float>(a, ref, out, s);
    case STORE_F16: return launch_stream_state_t<27, F16Dev>(a, ref, out, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace cflbm
