// Launches for waveform model 1 (IMRPhenomD); the launch code is shared with the other models.
#define GWF_MODEL 1
#include "gwf_run.cuh"

namespace gwf {

size_t setup_stride_m1() { return rec_stride<1>() + f32_stride<1>(); }
size_t core_bytes_m1() { return wave_bytes<1>(); }
cudaError_t launch_fisher_m1(const LaunchArgs& a) { return fisher_dispatch(a); }
cudaError_t launch_snr_m1(const LaunchArgs& a) { return snr_dispatch(a); }
cudaError_t launch_wave_m1(const LaunchArgs& a, const WaveOut& o) { return wave_dispatch(a, o); }
cudaError_t launch_group_m1(const LaunchArgs& a, const GroupDev& g) { return group_dispatch(a, g); }
cudaError_t launch_group64_m1(const LaunchArgs& a, const Group64& g) { return group64_dispatch(a, g); }
cudaError_t launch_snr_group64_m1(const LaunchArgs& a, const Group64& g) { return snr_group64_dispatch(a, g); }
cudaError_t launch_snr_group_f32_m1(const LaunchArgs& a, const Group64& g) { return snr_group_f32_dispatch(a, g); }

}  // namespace gwf
