// Launches for waveform model 3 (TaylorF2 with tidal terms, 13 Fisher parameters; FP64 only); the
// launch code is shared with the other models.
#define GWF_MODEL 3
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m3() { return rec_stride<3>(); }
size_t core_bytes_m3() { return wave_bytes<3>(); }
cudaError_t launch_fisher_m3(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m3(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m3(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }

}  // namespace gwf
