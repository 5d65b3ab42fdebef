// Host interface of the tensor-core network path (ves_nets_tc.cu).
#pragma once

#include <vector>

#include "ves_internal.h"

// Launch shape of one block's three kernels: warp groups per CTA and M = 64
// MMAs (for layers of at most 64 positions) in down and up1.
struct TcPlan {
  int nv;
  int ng_down, m64_down, ng_up1, m64_up1, ng_up2;
};

struct TcBlock {
  int geo[64];          // opaque block geometry (tcnet::Geo)
  int geo_bytes;
  int dsize, u1size, u2size;  // weight image bytes per group (down / up1 / up2 kernels)
  int mid_bytes;        // intermediates per (vesicle, group): down -> up1 -> up2
  size_t down_off, up1_off, up2_off;  // byte offsets of the block's images in the device buffer
  mutable std::vector<TcPlan> plans;  // autotuned launch shapes, one per vesicle count seen
};

// Build the per-group weight images of one block (30 reference parameter
// arrays, see ves_net_create) for sequence length L.
int tcnet_pack(const ves_net_block& b, int G, int L, const float* const* params, std::vector<unsigned char>& down,
               std::vector<unsigned char>& up1, std::vector<unsigned char>& up2, TcBlock& out);
// One block: x [nv][G*cin][L] -> out [nv][G*cout][L] (FP32), mid = scratch of
// (nv rounded up to a multiple of 4)*G*mid_bytes.
// autotune: on the first call for a vesicle count, time every launch shape
// that fits (warp groups per CTA, M = 64 MMAs on or off) of each kernel on
// this input and keep the fastest for later calls with that count (the
// stream is synchronised during the timing); otherwise the fixed rule.
int tcnet_run_block(const TcBlock& tb, int G, int nv, const unsigned char* d_down, const unsigned char* d_up1,
                    const unsigned char* d_up2, const float* x, float* out, unsigned char* mid,
                    VesDeviceStatus* st, cudaStream_t s, bool autotune = false);
