// Launches for waveform model 5 (eccentric TaylorF2, 12 Fisher parameters; FP64 only); the launch code is shared with the
// other models.
#define GWF_MODEL 5
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m5() { return rec_stride<5>(); }
size_t core_bytes_m5() { return wave_bytes<5>(); }
cudaError_t launch_fisher_m5(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m5(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m5(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }

}  // namespace gwf
