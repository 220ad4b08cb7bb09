// Launches for waveform model 6 (tidal eccentric TaylorF2, 14 Fisher parameters; FP64 only); the launch code is shared with the
// other models.
#define GWF_MODEL 6
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m6() { return rec_stride<6>(); }
size_t core_bytes_m6() { return wave_bytes<6>(); }
cudaError_t launch_fisher_m6(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m6(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m6(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }

}  // namespace gwf
