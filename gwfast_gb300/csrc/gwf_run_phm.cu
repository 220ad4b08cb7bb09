// Launches for waveform model 2 (IMRPhenomHM); the launch code is shared with the other models.
#define GWF_MODEL 2
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m2() { return rec_stride<2>() + f32_stride<2>(); }
size_t core_bytes_m2() { return wave_bytes<2>(); }
cudaError_t launch_fisher_m2(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m2(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m2(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }
cudaError_t launch_group_m2(const LaunchArgs& a, const GroupDev& g) { return group_dispatch(a, g); }
cudaError_t launch_group64_m2(const LaunchArgs& a, const Group64& g) { return group64_dispatch(a, g); }
cudaError_t launch_snr_group64_m2(const LaunchArgs& a, const Group64& g) { return snr_group64_dispatch(a, g); }
cudaError_t launch_snr_group_f32_m2(const LaunchArgs& a, const Group64& g) { return snr_group_f32_dispatch(a, g); }

}  // namespace gwf
