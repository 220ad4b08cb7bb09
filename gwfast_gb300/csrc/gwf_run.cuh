// Launch sequences of one waveform model. Each gwf_run_*.cu (one per model id) defines GWF_MODEL
// and includes this file, so the models compile as separate translation units in parallel.
//
// Per chunk of events: the per-event set-up kernel (FP64 records; a gathered batch whose records
// an earlier pass of the call left in scratch copies them instead), for the FP32 form the FP32
// record kernel, then either the classic Fisher/SNR kernel (one CTA per event) or, when the
// launch asks for segments, the segment scan, the persistent work-stealing Fisher kernel and the
// per-event reduction of the segment partials.
#include "gwf_launch.h"

namespace gwf {

namespace {

constexpr int M = GWF_MODEL;

unsigned char* scratch32_of(const LaunchArgs& a) { return a.scratch + (size_t)a.cap_events * rec_stride<M>(); }

// set-up records idx[i] of src -> record i of dst, in 16-byte words (rec_stride is a multiple of 16)
__global__ void copy_records_kernel(const uint4* __restrict__ src, const long long* __restrict__ idx, long long cnt,
                                    uint4* __restrict__ dst) {
  constexpr long long W = (long long)(rec_stride<M>() / 16);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt * W) return;
  const long long i = t / W;
  dst[t] = src[idx[i] * W + (t - i * W)];
}

template <class MAIN>
cudaError_t chunked(const LaunchArgs& a, bool f32, MAIN main) {
  for (long long n0 = 0; n0 < a.ev.N; n0 += kChunk) {
    EvBatch ev = a.ev;
    ev.n0 = n0;
    const long long cnt = (a.ev.N - n0) < kChunk ? (a.ev.N - n0) : kChunk;
    const int epw = ev_lanes(cnt);
    const unsigned nb = ev_blocks(cnt, epw);
    if (a.timer) {
      const cudaError_t et = a.timer->begin(a.stream, GWF_KT_SETUP);
      if (et != cudaSuccess) return et;
    }
    if (a.rec_src && a.core_idx) {
      const long long words = cnt * (long long)(rec_stride<M>() / 16);
      copy_records_kernel<<<(unsigned)((words + 255) / 256), 256, 0, a.stream>>>(
          reinterpret_cast<const uint4*>(a.rec_src), a.core_idx + n0, cnt, reinterpret_cast<uint4*>(a.scratch));
      if constexpr (M < 3) {   // (only the detector groups of the FP32 forms share records)
        if (a.rec_patch_proj) proj_patch_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, a.det, a.scratch, cnt, epw);
      }
    } else {
      setup_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, a.det, a.wf, a.qnm, a.nq, a.scratch, cnt, a.core, a.core_mode,
                                                     a.core_idx, epw);
    }
    if (a.core_done && a.core_mode == 1) {
      const cudaError_t er = cudaEventRecord(a.core_done, a.stream);
      if (er != cudaSuccess) return er;
    }
    if constexpr (M < 3) {   // (the tidal models have no FP32 form)
      const int repw = ev_lanes(cnt, kRecWarpsPerSM);
      if (f32)
        setup_f32_kernel<M><<<ev_blocks(cnt, repw), kEvBlock, 0, a.stream>>>(a.det, a.scratch, scratch32_of(a), cnt,
                                                                             a.det.shape == 1 ? 2 : 1, a.det.earth, repw);
    }
    if (a.timer) {
      const cudaError_t et = a.timer->end(a.stream);
      if (et != cudaSuccess) return et;
    }
    const cudaError_t e = main(ev, cnt);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

SegInfo seg_info(const LaunchArgs& a) {
  SegInfo si;
  si.off = a.seg_off;
  si.counter = a.seg_ctr;
  si.partial = a.seg_part;
  si.cap = a.seg_cap;
  si.seg = a.seg;
  si.overflow = a.seg_ovf;
  return si;
}

// segmented launch of one chunk: scan, persistent kernel, reduction
template <int NG, class KSEG>
cudaError_t seg_chunk(const LaunchArgs& a, const EvBatch& ev, long long cnt, KSEG ks, const unsigned char* kscratch,
                      int smem, int grid, const double* rec, long long stride_d) {
  cudaError_t e = a.timer ? a.timer->begin(a.stream, GWF_KT_SEGMENTED) : cudaSuccess;
  if (e != cudaSuccess) return e;
  seg_scan_kernel<M><<<1, 1024, 0, a.stream>>>(a.scratch, cnt, a.seg, a.seg_off);
  e = cudaMemsetAsync(a.seg_ctr, 0, sizeof(unsigned long long), a.stream);
  if (e != cudaSuccess) return e;
  const SegInfo si = seg_info(a);
  // no more CTAs than items (seg_cap bounds them): a small batch then spreads over distinct SMs
  // instead of stacking on the first SMs of a full persistent grid
  if (a.seg_cap > 0 && a.seg_cap < grid) grid = (int)a.seg_cap;
  ks<<<grid, kThreads, smem, a.stream>>>(ev, a.det, kscratch, cnt, si, (a.out_sd_arm || a.out_sd_det) ? 1 : 0);
  gram_reduce_kernel<NG><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev.n0, ev.N, cnt, si, rec, stride_d, a.out_arm,
                                                                   a.out_det, a.out_sd_arm, a.out_sd_det, a.accum);
  e = cudaGetLastError();
  if (e == cudaSuccess && a.timer) e = a.timer->end(a.stream);
  return e;
}

template <class K>
cudaError_t persist_grid(K k, int smem, int* grid) {
  int occ = 0;
  const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kThreads, smem);
  if (e != cudaSuccess) return e;
  *grid = (occ > 0 ? occ : 1) * device_sms();
  return cudaSuccess;
}

template <bool EARTH, int NARM, int NG>
cudaError_t fisher_one(const LaunchArgs& a) {
  const int smem = kWarps * NG * (np_of<M>() + 1) * kSR64 * (int)sizeof(cd);
  if (a.seg <= 0 || M >= 3) {
    auto k = fisher_kernel<M, EARTH, NARM, NG>;
    cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return err;
    return chunked(a, false, [&](const EvBatch& ev, long long cnt) {
      if (a.timer) a.timer->begin(a.stream, GWF_KT_FISHER_F64);
      k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, a.det, a.scratch, a.out_arm, a.out_det, a.out_sd_arm,
                                                     a.out_sd_det, a.accum);
      return a.timer ? a.timer->end(a.stream) : cudaSuccess;
    });
  }
  if constexpr (M >= 3) {
    return cudaErrorNotSupported;   // not reached: the tidal models always run one CTA per event
  } else {
    auto ks = fisher_seg_kernel<M, EARTH, NARM, NG>;
    cudaError_t err = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int grid = 0;
    if (err == cudaSuccess) err = persist_grid(ks, smem, &grid);
    if (err != cudaSuccess) return err;
    return chunked(a, false, [&](const EvBatch& ev, long long cnt) {
      return seg_chunk<NG>(a, ev, cnt, ks, a.scratch, smem, grid, nullptr, 0);
    });
  }
}

template <bool EARTH, int NARM, int NG>
cudaError_t fisher_one_f32(const LaunchArgs& a) {
  const int smem = kWarps * NG * 12 * kSR * (int)sizeof(int2);
  unsigned char* s32 = scratch32_of(a);
  if (a.seg <= 0) {
    auto k = fisher_kernel_f32<M, EARTH, NARM, NG>;
    cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return err;
    return chunked(a, true, [&](const EvBatch& ev, long long cnt) {
      if (a.timer) a.timer->begin(a.stream, GWF_KT_FISHER_F32);
      k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, a.det, s32, a.out_arm, a.out_det, a.out_sd_arm, a.out_sd_det,
                                                     a.accum);
      return a.timer ? a.timer->end(a.stream) : cudaSuccess;
    });
  }
  auto ks = fisher_seg_kernel_f32<M, EARTH, NARM, NG>;
  cudaError_t err = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int grid = 0;
  if (err == cudaSuccess) err = persist_grid(ks, smem, &grid);
  if (err != cudaSuccess) return err;
  // Gram scale, psi-column sign and chi1 column coefficient lead each FP32 record
  const double* rec0 = reinterpret_cast<const double*>(s32);
  const long long stride_d = (long long)(f32_stride<M>() / sizeof(double));
  return chunked(a, true, [&](const EvBatch& ev, long long cnt) {
    return seg_chunk<NG>(a, ev, cnt, ks, s32, smem, grid, rec0, stride_d);
  });
}

template <bool EARTH, int NARM>
cudaError_t snr_one(const LaunchArgs& a) {
  return chunked(a, false, [&](const EvBatch& ev, long long cnt) {
    snr_kernel<M, EARTH, NARM><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev, a.det, a.scratch, a.out_arm, a.out_det,
                                                                          a.accum);
    return cudaSuccess;
  });
}

cudaError_t fisher_dispatch(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.precision == 1) {
    if constexpr (M >= 3) {
      return cudaErrorNotSupported;
    } else {
      if (a.det.earth) {
        if (!tri) return fisher_one_f32<true, 1, 1>(a);
        return a.per_arm ? fisher_one_f32<true, 2, 3>(a) : fisher_one_f32<true, 2, 2>(a);
      }
      if (!tri) return fisher_one_f32<false, 1, 1>(a);
      return a.per_arm ? fisher_one_f32<false, 2, 3>(a) : fisher_one_f32<false, 2, 2>(a);
    }
  }
  if (a.det.earth) {
    if (!tri) return fisher_one<true, 1, 1>(a);
    return a.per_arm ? fisher_one<true, 2, 3>(a) : fisher_one<true, 2, 2>(a);
  }
  if (!tri) return fisher_one<false, 1, 1>(a);
  return a.per_arm ? fisher_one<false, 2, 3>(a) : fisher_one<false, 2, 2>(a);
}

#if GWF_MODEL < 3
template <bool EARTH, int NARM>
cudaError_t snr_one_f32(const LaunchArgs& a) {
  unsigned char* s32 = scratch32_of(a);
  return chunked(a, true, [&](const EvBatch& ev, long long cnt) {
    snr_kernel_f32<M, EARTH, NARM><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev, a.det, s32, a.out_arm, a.out_det,
                                                                              a.accum);
    return cudaSuccess;
  });
}
#endif

cudaError_t snr_dispatch(const LaunchArgs& a) {
  const bool tri = a.det.shape == 1;
  if (a.precision == 1) {
#if GWF_MODEL < 3
    if (a.det.earth) return tri ? snr_one_f32<true, 2>(a) : snr_one_f32<true, 1>(a);
    return tri ? snr_one_f32<false, 2>(a) : snr_one_f32<false, 1>(a);
#else
    return cudaErrorNotSupported;
#endif
  }
  if (a.det.earth) return tri ? snr_one<true, 2>(a) : snr_one<true, 1>(a);
  return tri ? snr_one<false, 2>(a) : snr_one<false, 1>(a);
}

// a group of detectors sharing the grid (network total, FP32 form): per chunk, the set-up of each
// detector into its own scratch slice, then one launch over all of them
template <bool EARTH, bool TRI>
cudaError_t group_one(const LaunchArgs& a, GroupDev g) {
  const int smem = kWarps * 12 * kSR * (int)sizeof(int2);
  auto k = fisher_group_kernel_f32<M, EARTH, TRI>;
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (err != cudaSuccess) return err;
  const long long chunk = a.cap_events;
  const size_t stride = rec_stride<M>() + f32_stride<M>();
  g.slice = (long long)(chunk * stride);
  for (long long n0 = 0; n0 < a.ev.N; n0 += chunk) {
    EvBatch ev = a.ev;
    ev.n0 = n0;
    const long long cnt = (a.ev.N - n0) < chunk ? (a.ev.N - n0) : chunk;
    const int epw = ev_lanes(cnt);
    const unsigned nb = ev_blocks(cnt, epw);
    if (a.timer) {
      err = a.timer->begin(a.stream, GWF_KT_SETUP);
      if (err != cudaSuccess) return err;
    }
    for (int d = 0; d < g.nd; ++d) {
      unsigned char* sc = a.scratch + (size_t)d * chunk * stride;
      unsigned char* s32 = sc + (size_t)chunk * rec_stride<M>();
      if (d > 0) {   // same grid and model record as detector 0: only the projection is its own
        proj_f32_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, g.det[d], s32, cnt, g.det[d].shape == 1 ? 2 : 1,
                                                          g.det[d].earth, epw);
        continue;
      }
      setup_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, g.det[d], a.wf, a.qnm, a.nq, sc, cnt, a.core, a.core_mode,
                                                     nullptr, epw);
      if (a.core_done && a.core_mode == 1) {
        err = cudaEventRecord(a.core_done, a.stream);
        if (err != cudaSuccess) return err;
      }
      const int repw = ev_lanes(cnt, kRecWarpsPerSM);
      setup_f32_kernel<M><<<ev_blocks(cnt, repw), kEvBlock, 0, a.stream>>>(g.det[d], sc, s32, cnt,
                                                                           g.det[d].shape == 1 ? 2 : 1, g.det[d].earth, repw);
    }
    if (a.timer) {
      err = a.timer->end(a.stream);
      if (err == cudaSuccess) err = a.timer->begin(a.stream, GWF_KT_GROUP_F32);
      if (err != cudaSuccess) return err;
    }
    k<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, g, a.scratch + (size_t)chunk * rec_stride<M>(), a.out_det, a.accum);
    err = cudaGetLastError();
    if (err == cudaSuccess && a.timer) err = a.timer->end(a.stream);
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

// FP32 SNR of a group of detectors on one grid (the set-up as group_one: detector 0's FP64 and FP32
// records, the others' projection only), then one launch over the group
template <bool EARTH, bool TRI>
cudaError_t snr_group_one_f32(const LaunchArgs& a, const Group64& G) {
  if constexpr (M >= 3) {
    return cudaErrorNotSupported;
  } else {
    const long long chunk = a.cap_events;
    const size_t stride = rec_stride<M>() + f32_stride<M>();
    GroupSNR32 g;
    g.nd = G.nd;
    g.slice = (long long)(chunk * stride);
    for (int d = 0; d < G.nd; ++d) {
      g.det[d] = G.det[d];
      g.out_arm[d] = G.out_arm[d];
      g.sr[d] = G.det[0].psd_scale / G.det[d].psd_scale;
      g.same_psd[d] = G.same_psd[d];
    }
    for (long long n0 = 0; n0 < a.ev.N; n0 += chunk) {
      EvBatch ev = a.ev;
      ev.n0 = n0;
      const long long cnt = (a.ev.N - n0) < chunk ? (a.ev.N - n0) : chunk;
      const int epw = ev_lanes(cnt);
      const unsigned nb = ev_blocks(cnt, epw);
      for (int d = 0; d < G.nd; ++d) {
        unsigned char* sc = a.scratch + (size_t)d * chunk * stride;
        unsigned char* s32 = sc + (size_t)chunk * rec_stride<M>();
        const int narm = G.det[d].shape == 1 ? 2 : 1;
        if (d > 0) {
          proj_f32_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, G.det[d], s32, cnt, narm, G.det[d].earth, epw);
          continue;
        }
        setup_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, G.det[0], a.wf, a.qnm, a.nq, sc, cnt, a.core, a.core_mode,
                                                       nullptr, epw);
        if (a.core_done && a.core_mode == 1) {
          const cudaError_t e = cudaEventRecord(a.core_done, a.stream);
          if (e != cudaSuccess) return e;
        }
        const int repw = ev_lanes(cnt, kRecWarpsPerSM);
        setup_f32_kernel<M><<<ev_blocks(cnt, repw), kEvBlock, 0, a.stream>>>(G.det[0], sc, s32, cnt, narm, G.det[0].earth,
                                                                             repw);
      }
      snr_group_kernel_f32<M, EARTH, TRI><<<(unsigned)cnt, kThreads, 0, a.stream>>>(
          ev, g, a.scratch + (size_t)chunk * rec_stride<M>(), a.out_det, a.accum);
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
}

cudaError_t snr_group_f32_dispatch(const LaunchArgs& a, const Group64& G) {
  bool tri = false;
  for (int d = 0; d < G.nd; ++d) tri |= G.det[d].shape == 1;
  if (tri) return a.det.earth ? snr_group_one_f32<true, true>(a, G) : snr_group_one_f32<false, true>(a, G);
  return a.det.earth ? snr_group_one_f32<true, false>(a, G) : snr_group_one_f32<false, false>(a, G);
}

cudaError_t group_dispatch(const LaunchArgs& a, const GroupDev& g) {
  if constexpr (M >= 3) return cudaErrorNotSupported;
  else {
    bool tri = false;
    for (int d = 0; d < g.nd; ++d) tri |= g.det[d].shape == 1;
    if (tri) return a.det.earth ? group_one<true, true>(a, g) : group_one<false, true>(a, g);
    return a.det.earth ? group_one<true, false>(a, g) : group_one<false, false>(a, g);
  }
}

// records of events [ev.n0, ev.n0 + cnt) for each member of an FP64 group: detector 0 runs the set-up
// (or, for a gathered batch, copies the first pass's records), the others get their projection header
// only, which is all the group kernels read of them
cudaError_t group64_records(const LaunchArgs& a, const Group64& G, const EvBatch& ev, long long cnt, int epw,
                            unsigned nb) {
  for (int d = 0; d < G.nd; ++d) {
    unsigned char* sc = G.scratch[d];
    if (G.rec_src[d] && a.core_idx) {
      const long long words = cnt * (long long)(rec_stride<M>() / 16);
      copy_records_kernel<<<(unsigned)((words + 255) / 256), 256, 0, a.stream>>>(
          reinterpret_cast<const uint4*>(G.rec_src[d]), a.core_idx + ev.n0, cnt, reinterpret_cast<uint4*>(sc));
      if (G.patch[d]) proj_patch_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, G.det[d], sc, cnt, epw);
    } else if (d == 0) {
      setup_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, G.det[0], a.wf, a.qnm, a.nq, sc, cnt, a.core, a.core_mode,
                                                     a.core_idx, epw);
      if (a.core_done && a.core_mode == 1) {
        const cudaError_t err = cudaEventRecord(a.core_done, a.stream);
        if (err != cudaSuccess) return err;
      }
    } else {
      proj_patch_kernel<M><<<nb, kEvBlock, 0, a.stream>>>(ev, G.det[d], sc, cnt, epw);
    }
  }
  return cudaGetLastError();
}

// FP64 network total of a group of detectors on one grid: per chunk each member's records (detector
// 0: the set-up, or for a gathered batch a copy of the first pass's records; the others: their
// projection header only, which is all the group kernel reads of them), then one launch over the
// group, classic or segmented. TRI: a member is a triangle (a second set of staging rows).
template <bool EARTH, bool TRI>
cudaError_t group64_one(const LaunchArgs& a, const Group64& G) {
  if constexpr (np_of<M>() != NP) {
    return cudaErrorNotSupported;
  } else {
    const int smem = kWarps * (TRI ? 2 : 1) * (np_of<M>() + 1) * kSR64 * (int)sizeof(cd);
    GroupDev64 g;
    g.nd = G.nd;
    for (int d = 0; d < G.nd; ++d) {
      g.det[d] = G.det[d];
      g.rec[d] = G.scratch[d];
      g.same_psd[d] = G.same_psd[d];
    }
    auto kc = fisher_group_kernel64<M, EARTH, TRI>;
    auto ks = fisher_group_seg_kernel64<M, EARTH, TRI>;
    cudaError_t err = cudaFuncSetAttribute(kc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err == cudaSuccess) err = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int grid = 0;
    if (err == cudaSuccess && a.seg > 0) err = persist_grid(ks, smem, &grid);
    if (err != cudaSuccess) return err;
    const long long chunk = a.cap_events;
    for (long long n0 = 0; n0 < a.ev.N; n0 += chunk) {
      EvBatch ev = a.ev;
      ev.n0 = n0;
      const long long cnt = (a.ev.N - n0) < chunk ? (a.ev.N - n0) : chunk;
      const int epw = ev_lanes(cnt);
      const unsigned nb = ev_blocks(cnt, epw);
      if (a.timer && (err = a.timer->begin(a.stream, GWF_KT_SETUP)) != cudaSuccess) return err;
      if ((err = group64_records(a, G, ev, cnt, epw, nb)) != cudaSuccess) return err;
      if (a.timer && (err = a.timer->end(a.stream)) != cudaSuccess) return err;
      if (a.seg > 0) {
        if (a.timer && (err = a.timer->begin(a.stream, GWF_KT_SEGMENTED)) != cudaSuccess) return err;
        seg_scan_kernel<M><<<1, 1024, 0, a.stream>>>(G.scratch[0], cnt, a.seg, a.seg_off);
        if ((err = cudaMemsetAsync(a.seg_ctr, 0, sizeof(unsigned long long), a.stream)) != cudaSuccess) return err;
        const SegInfo si = seg_info(a);
        const int gr = (a.seg_cap > 0 && a.seg_cap < grid) ? (int)a.seg_cap : grid;
        ks<<<gr, kThreads, smem, a.stream>>>(ev, g, cnt, si);
        gram_reduce_kernel<1><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev.n0, ev.N, cnt, si, nullptr, 0, nullptr,
                                                                        a.out_det, nullptr, nullptr, a.accum);
      } else {
        if (a.timer && (err = a.timer->begin(a.stream, GWF_KT_FISHER_F64)) != cudaSuccess) return err;
        kc<<<(unsigned)cnt, kThreads, smem, a.stream>>>(ev, g, a.out_det, a.accum);
      }
      err = cudaGetLastError();
      if (err == cudaSuccess && a.timer) err = a.timer->end(a.stream);
      if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
  }
}

// FP64 SNR of a group of detectors on one grid: per chunk the members' records, then one launch
template <bool EARTH, bool TRI>
cudaError_t snr_group64_one(const LaunchArgs& a, const Group64& G) {
  if constexpr (np_of<M>() != NP) {
    return cudaErrorNotSupported;
  } else {
    GroupSNR64 g;
    g.nd = G.nd;
    for (int d = 0; d < G.nd; ++d) {
      g.det[d] = G.det[d];
      g.rec[d] = G.scratch[d];
      g.out_arm[d] = G.out_arm[d];
      g.same_psd[d] = G.same_psd[d];
    }
    const long long chunk = a.cap_events;
    for (long long n0 = 0; n0 < a.ev.N; n0 += chunk) {
      EvBatch ev = a.ev;
      ev.n0 = n0;
      const long long cnt = (a.ev.N - n0) < chunk ? (a.ev.N - n0) : chunk;
      const int epw = ev_lanes(cnt);
      cudaError_t err = group64_records(a, G, ev, cnt, epw, ev_blocks(cnt, epw));
      if (err != cudaSuccess) return err;
      snr_group_kernel64<M, EARTH, TRI><<<(unsigned)cnt, kThreads, 0, a.stream>>>(ev, g, a.out_det, a.accum);
      if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    return cudaSuccess;
  }
}

cudaError_t snr_group64_dispatch(const LaunchArgs& a, const Group64& G) {
  bool tri = false;
  for (int d = 0; d < G.nd; ++d) tri |= G.det[d].shape == 1;
  if (tri) return a.det.earth ? snr_group64_one<true, true>(a, G) : snr_group64_one<false, true>(a, G);
  return a.det.earth ? snr_group64_one<true, false>(a, G) : snr_group64_one<false, false>(a, G);
}

cudaError_t group64_dispatch(const LaunchArgs& a, const Group64& G) {
  bool tri = false;
  for (int d = 0; d < G.nd; ++d) tri |= G.det[d].shape == 1;
  if (tri) return a.det.earth ? group64_one<true, true>(a, G) : group64_one<false, true>(a, G);
  return a.det.earth ? group64_one<true, false>(a, G) : group64_one<false, false>(a, G);
}

template <bool EARTH, int NARM>
cudaError_t wave_one(const LaunchArgs& a, const WaveOut& o) {
  EvBatch ev = a.ev;
  ev.n0 = o.n0;
  const int epw = ev_lanes(o.cnt);
  setup_kernel<M><<<ev_blocks(o.cnt, epw), kEvBlock, 0, a.stream>>>(ev, a.det, a.wf, a.qnm, a.nq, a.scratch, o.cnt,
                                                                    nullptr, 0, nullptr, epw);
  wave_out_kernel<M, EARTH, NARM><<<(unsigned)o.cnt, kThreads, 0, a.stream>>>(ev, a.det, a.scratch, o);
  return cudaGetLastError();
}

cudaError_t wave_dispatch(const LaunchArgs& a, const WaveOut& o) {
  if (o.cnt <= 0) return cudaSuccess;
  const bool tri = a.det.shape == 1;
  if (a.det.earth) return tri ? wave_one<true, 2>(a, o) : wave_one<true, 1>(a, o);
  return tri ? wave_one<false, 2>(a, o) : wave_one<false, 1>(a, o);
}

}  // namespace

}  // namespace gwf
