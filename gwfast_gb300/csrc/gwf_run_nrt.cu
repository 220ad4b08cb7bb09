// Launches for waveform model 4 (IMRPhenomD_NRTidalv2, 13 Fisher parameters; FP64 only); the launch
// code is shared with the other models.
#define GWF_MODEL 4
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m4() { return rec_stride<4>(); }
size_t core_bytes_m4() { return wave_bytes<4>(); }
cudaError_t launch_fisher_m4(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m4(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m4(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }

}  // namespace gwf
