// Launches for waveform model 0 (TaylorF2); the launch code is shared with the other models.
#define GWF_MODEL 0
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m0() { return rec_stride<0>() + f32_stride<0>(); }
size_t core_bytes_m0() { return wave_bytes<0>(); }
cudaError_t launch_fisher_m0(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m0(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m0(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }
cudaError_t launch_group_m0(const LaunchArgs& a, const GroupDev& g) { return group_dispatch(a, g); }
cudaError_t launch_group64_m0(const LaunchArgs& a, const Group64& g) { return group64_dispatch(a, g); }
cudaError_t launch_snr_group64_m0(const LaunchArgs& a, const Group64& g) { return snr_group64_dispatch(a, g); }
cudaError_t launch_snr_group_f32_m0(const LaunchArgs& a, const Group64& g) { return snr_group_f32_dispatch(a, g); }

}  // namespace gwf
