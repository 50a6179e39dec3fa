// D2Q9 instantiations of the fused sweep (see sweep.cuh).
#include "sweep.cuh"

namespace cflbm {

cudaError_t launch_sweep_q9(int store, int compute, const SweepArgs &a, cudaStream_t s) {
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_sweep_t<9, double, df64, 4>(a, s) : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_sweep_t<9, double, double, 4>(a, s);
      case STORE_F32: return launch_sweep_t<9, float, double, 4>(a, s);
      case STORE_F16: return launch_sweep_t<9, F16Dev, double, 4>(a, s);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_sweep_t<9, double, float, 4>(a, s);
      case STORE_F32: return launch_sweep_t<9, float, float, 4>(a, s);
      case STORE_F16: return launch_sweep_t<9, F16Dev, float, 4>(a, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_sweep_channel_q9(int store, int compute, const SweepArgs &a,
                                     cudaStream_t s, const SweepFork *fk) {
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_sweep_channel_t<9, double, df64, 4, 2>(a, s, fk)
                              : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_sweep_channel_t<9, double, double, 4, 2>(a, s, fk);
      case STORE_F32: return launch_sweep_channel_t<9, float, double, 4, 2>(a, s, fk);
      case STORE_F16: return launch_sweep_channel_t<9, F16Dev, double, 4, 2>(a, s, fk);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_sweep_channel_t<9, double, float, 8, 4>(a, s, fk);
      case STORE_F32: return launch_sweep_channel_t<9, float, float, 8, 4>(a, s, fk);
      case STORE_F16: return launch_sweep_channel_t<9, F16Dev, float, 8, 4>(a, s, fk);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_macros_channel_q9(int store, int compute, const SweepArgs &a,
                                      cudaStream_t s) {
  if (compute == COMPUTE_DF64)
    return store == STORE_F64 ? launch_macros_channel_t<9, double, df64>(a, s)
                              : cudaErrorInvalidValue;
  if (compute == COMPUTE_F64) {
    switch (store) {
      case STORE_F64: return launch_macros_channel_t<9, double, double>(a, s);
      case STORE_F32: return launch_macros_channel_t<9, float, double>(a, s);
      case STORE_F16: return launch_macros_channel_t<9, F16Dev, double>(a, s);
    }
  } else {
    switch (store) {
      case STORE_F64: return launch_macros_channel_t<9, double, float>(a, s);
      case STORE_F32: return launch_macros_channel_t<9, float, float>(a, s);
      case STORE_F16: return launch_macros_channel_t<9, F16Dev, float>(a, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_stream_state_q9(int store, const SweepArgs &a, bool ref, double *out,
                                    cudaStream_t s) {
  switch (store) {
    case STORE_F64: return launch_stream_state_t<9, double>(a, ref, out, s);
    case STORE_F32: return launch_stream_state_t<9, float>(a, ref, out, s);
    case STORE_F16: return launch_stream_state_t<9, F16Dev>(a, ref, out, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace cflbm
