// Per-epoch ConnGrowth pass and recorder, on the device.
//
//   k_growth_radii     rates = spikeCount / T; radii += T * rho * outgrowth      (O(N))
//   k_growth_existing  W of every in-use synapse from the overlap area of its pair (O(S))
//   k_growth_rmax      the largest radius (one CTA)
//   k_growth_add       one CTA per destination scans the sources in ascending order (on the grid
//                      layout only the window within the largest radius), computes the frontier
//                      distance / overlap area, and appends the new synapses in source order after
//                      the row's in-use prefix            (O(N^2) pairs, no N^2 storage)
//   k_out_count/scan/fill  outgoing CSR rebuild per delay class (createSynapseImap)
//   k_record_epoch     recorder histograms, rates/radii history, radius clamp, spike-count roll
#include "bg3_internal.cuh"

namespace bg3 {

// ConnGrowth::updateConns (Connections/ConnGrowth.cpp:295-311).
__global__ void k_growth_radii(const NetDev *nets)
{
    const NetDev &n = nets[0];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n.N) return;
    float T = n.epoch_duration;
    const int cnt = n.spikeCount[i];
    float rate = (float)cnt / T;
    n.rates[i] = rate;
    // expf of the host library for every possible count, evaluated there in this order
    float e = (cnt >= 0 && cnt <= n.max_spikes) ? n.grow_exp[cnt]
                                                : exp_cr((n.g_epsilon - rate / n.g_max_rate) / n.g_beta);
    float og = 1.0f - 2.0f / (e + 1.0f);
    float trho = T * n.g_rho;
    n.radii[i] = n.radii[i] + trho * og;
}

// Frontier distance and overlap area of the pair (i = source, j = dest)
// (Connections/ConnGrowth.cpp:319-376; dist from Layouts/Layout.cpp:54-69).  Returns 0 for pairs
// that do not overlap.  Double where the reference promotes (2.0 * r * len, 2.0 * angle, 0.5 *).
__device__ __forceinline__ float pair_area(float xi, float yi, float ri, float xj, float yj,
                                           float rj)
{
    float dx = xi - xj, dy = yi - yj;
    float len2 = dx * dx + dy * dy;
    float len = sqrtf(len2);
    float delta = len - (ri + rj);
    if (!(delta < 0.0f)) return 0.0f;
    float rmin = fminf(ri, rj), rmax = fmaxf(ri, rj);
    if (len + rmin <= rmax) {
        const float pi = 3.1415926536f;  // Utils/Global.cpp:90
        return pi * rmin * rmin;
    }
    float r12 = ri * ri, r22 = rj * rj;
    float cosCBA = (float)((double)(r22 + len2 - r12) / (2.0 * (double)rj * (double)len));
    float angCBA = acos_cr(cosCBA);
    float angCBD = (float)(2.0 * (double)angCBA);
    float cosCAB = (float)((double)(r12 + len2 - r22) / (2.0 * (double)ri * (double)len));
    float angCAB = acos_cr(cosCAB);
    float angCAD = (float)(2.0 * (double)angCAB);
    return (float)(0.5 * (double)(r22 * (angCBD - sin_cr(angCBD)) + r12 * (angCAD - sin_cr(angCAD))));
}

// Layout::synType (Layouts/Layout.cpp:129-140): II 0, IE 1, EI 2, EE 3.
__device__ __forceinline__ int syn_type(int8_t ts, int8_t td)
{
    return (ts == 1) ? ((td == 1) ? 0 : 1) : ((td == 1) ? 2 : 3);
}
__device__ __forceinline__ float syn_sign(int type) { return (type <= 1) ? -1.0f : 1.0f; }

// Weight update of existing synapses (ConnGrowth.cpp:420-438):
// W = area * synSign(type) * SYNAPSE_STRENGTH_ADJUSTMENT (1.0e-8).
__global__ void k_growth_existing(const NetDev *nets)
{
    const NetDev &n = nets[0];
    size_t total = (size_t)n.Np * n.Mq * 4;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
         p += (size_t)gridDim.x * blockDim.x) {
        int d, k;
        pos_slot(p, n.Mq, k, d);
        if (d >= n.N || k >= (int)n.count[d]) continue;
        int s = n.src[p];
        float a = pair_area(n.xloc[s], n.yloc[s], n.radii[s], n.xloc[d], n.yloc[d], n.radii[d]);
        if (a < 0.0f) set_err(n, ERR_NEGATIVE_AREA);  // the reference would erase (area >= 0)
        n.ev[p].W = a * syn_sign(n.stype[p]) * 1.0e-8f;
    }
}

// The largest radius after the epoch's radius update (negative radii count as 0), for the
// overlap scan's window: one CTA.
__global__ void __launch_bounds__(1024) k_growth_rmax(const NetDev *nets)
{
    const NetDev &n = nets[0];
    __shared__ float wmax[32];
    float m = 0.0f;
    for (int i = threadIdx.x; i < n.N; i += blockDim.x) m = fmaxf(m, n.radii[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) *n.grow_rmax = m;
    }
}

// The sources a destination's overlap scan visits, in ascending index order: all N, or on the
// reference's grid layout only the square window of rows and columns within K of the
// destination, where K + 1 > fl(rmax + r_d).  Outside it |dx| or |dy| >= fl(rmax + r_d), so
// len = sqrtf(dx^2 + dy^2) >= fl(r_s + r_d) (grid coordinates are whole numbers, their squares and
// sums exact; sqrtf and rounding are monotone) and the pair's delta = len - (r_s + r_d) is not
// negative: no overlap, exactly as the full scan finds.  Candidate c is source
// (y0 + c / cw) * W + x0 + c % cw.
struct ScanWindow {
    int x0, y0, cw, count;  // cw = 0: the full scan (candidate c is source c)
};
__device__ __forceinline__ ScanWindow scan_window(const NetDev &n, int d, float rd)
{
    ScanWindow w = {0, 0, 0, n.N};
    const int W = n.grid_w, H = n.grid_h;
    if (W <= 0 || H <= 0 || (long long)W * H != (long long)n.N) return w;
    const float bound = *n.grow_rmax + rd;
    if (!(bound >= 0.0f) || bound > (float)(W + H)) return w;  // NaN, or a window wider than the grid
    const int K = (int)ceilf(bound) - 1;
    if (K < 0) {
        w.count = 0;
        return w;
    }
    const int xd = d % W, yd = d / W;
    w.x0 = max(0, xd - K);
    w.y0 = max(0, yd - K);
    w.cw = min(W - 1, xd + K) - w.x0 + 1;
    w.count = w.cw * (min(H - 1, yd + K) - w.y0 + 1);
    return w;
}
__device__ __forceinline__ int window_source(const NetDev &n, const ScanWindow &w, int c)
{
    if (w.cw == 0) return c;
    return (w.y0 + c / w.cw) * n.grid_w + w.x0 + c % w.cw;
}

// New synapses (ConnGrowth.cpp:441-454, AllSynapses::addSynapse :357-377, create* of
// AllSpikingSynapses.cpp:192-240 / AllDSSynapses.cpp:180-218).  One CTA per destination, over
// the sources of its scan window in ascending order.
template <int ADD_THREADS>
__global__ void __launch_bounds__(ADD_THREADS) k_growth_add(const NetDev *nets)
{
    const NetDev &n = nets[0];
    extern __shared__ uint32_t existing[];  // N bits
    __shared__ int warp_cnt[ADD_THREADS / 32];
    __shared__ int s_count;
    const int d = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int words = (n.N + 31) / 32;
    for (int w = threadIdx.x; w < words; w += blockDim.x) existing[w] = 0u;
    if (threadIdx.x == 0) s_count = (int)n.count[d];
    __syncthreads();
    const int c0 = s_count;
    for (int k = threadIdx.x; k < c0; k += blockDim.x) {
        int s = n.src[slot_pos(k, d, n.Mq)];
        atomicOr(&existing[s >> 5], 1u << (s & 31));
    }
    __syncthreads();
    const float xd = n.xloc[d], yd = n.yloc[d], rd = n.radii[d];
    const int8_t td = n.ntype[d];
    const unsigned long long t = *n.step;
    const ScanWindow win = scan_window(n, d, rd);
    for (int base = 0; base < win.count; base += ADD_THREADS) {
        const int c = base + threadIdx.x;
        const int s = c < win.count ? window_source(n, win, c) : n.N;
        float a = 0.0f;
        bool add = false;
        if (s < n.N && s != d && !((existing[s >> 5] >> (s & 31)) & 1u)) {
            a = pair_area(n.xloc[s], n.yloc[s], n.radii[s], xd, yd, rd);
            add = a > 0.0f;
        }
        // most chunks add nothing (every pair beyond the radii): one barrier, no ordering
        if (!__syncthreads_or(add)) continue;
        unsigned m = __ballot_sync(0xffffffffu, add);
        if (lane == 0) warp_cnt[warp] = __popc(m);
        __syncthreads();
        int before = 0, tot = 0;
#pragma unroll
        for (int w = 0; w < ADD_THREADS / 32; w++) {
            int c = warp_cnt[w];
            if (w < warp) before += c;
            tot += c;
        }
        int cur = s_count;
        if (add) {
            int k = cur + before + __popc(m & ((1u << lane) - 1));
            if (k < n.max_syn) {
                size_t p = slot_pos(k, d, n.Mq);
                int type = syn_type(n.ntype[s], td);
                n.src[p] = s;
                n.stype[p] = (int8_t)type;
                n.psr[p] = 0.0f;
                // new slots hold class 0: set the slot's nibble (slots of other dests or rows
                // may share the word)
                atomicOr(&n.dcls[p >> 3], ((uint32_t)n.t_dcls[type] & 15u) << (4u * (uint32_t)(p & 7)));
                n.lcls[p] = (uint8_t)n.t_lcls[type];
                EvSlot e;
                e.W = a * syn_sign(type) * 1.0e-8f;
                e.dcls = (uint8_t)n.t_dcls[type];
                e.pcls = (uint8_t)n.t_pcls[type];
                e.pad0 = 0;
                e.pad1 = e.pad2 = 0u;
                e.u = n.t_u0;
                e.r = n.t_r0;
                e.last = BG3_NO_SPIKE32;
                e.born = (uint32_t)t;
                n.ev[p] = e;
            } else {
                set_err(n, ERR_ROW_FULL);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_count = min(cur + tot, n.max_syn);
        __syncthreads();
    }
    if (threadIdx.x == 0) n.count[d] = (uint32_t)s_count;
}

// ---- outgoing map (AllSynapses::createSynapseImap, Synapses/AllSynapses.cpp:223-293) ---------
// Grouped by delay class c then source i (index c * N + i); entries are plane slots.
__global__ void k_out_zero(const NetDev *nets)
{
    const NetDev &n = nets[0];
    int total = n.N * n.n_delays;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        n.outCount[i] = 0u;
        n.outFill[i] = 0u;
    }
}
__global__ void k_out_count(const NetDev *nets)
{
    const NetDev &n = nets[0];
    size_t total = (size_t)n.Np * n.Mq * 4;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
         p += (size_t)gridDim.x * blockDim.x) {
        int d, k;
        pos_slot(p, n.Mq, k, d);
        if (d < n.N && k < (int)n.count[d])
            atomicAdd(&n.outCount[(size_t)n.lcls[p] * n.N + n.src[p]], 1u);
    }
}
// exclusive scan of outCount into outBegin; one CTA of 1024 threads walks the table in chunks
__global__ void __launch_bounds__(1024) k_out_scan(const NetDev *nets)
{
    const NetDev &n = nets[0];
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int total = n.N * n.n_delays;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < total; b += 1024) {
        int i = b + threadIdx.x;
        uint32_t v = (i < total) ? n.outCount[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = wsum[lane], z = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            wsum[lane] = z - w;
        }
        __syncthreads();
        uint32_t c = carry;
        if (i < total) n.outBegin[i] = c + wsum[warp] + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + wsum[31] + x;
        __syncthreads();
    }
}
__global__ void k_out_fill(const NetDev *nets)
{
    const NetDev &n = nets[0];
    size_t total = (size_t)n.Np * n.Mq * 4;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total;
         p += (size_t)gridDim.x * blockDim.x) {
        int d, k;
        pos_slot(p, n.Mq, k, d);
        if (d >= n.N || k >= (int)n.count[d]) continue;
        size_t key = (size_t)n.lcls[p] * n.N + n.src[p];
        uint32_t slot = n.outBegin[key] + atomicAdd(&n.outFill[key], 1u);
        n.outMap[slot] = (uint32_t)p;
    }
}

// ---- recorder (Recorders/XmlRecorder.cpp:71-104, XmlGrowthRecorder.cpp:72-97,
//      Neurons/AllSpikingNeurons.cpp:77-86) ----------------------------------------------------
// XmlRecorder::compileHistories (Recorders/XmlRecorder.cpp:71-104) and, with growth, the
// XmlGrowthRecorder additions (XmlGrowthRecorder.cpp:72-97).
__global__ void k_record_epoch(const NetDev *nets, int epoch, bool growth)
{
    const NetDev &n = nets[0];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n.N) return;
    const int ms = n.max_spikes;
    const unsigned long long *h = n.history + (size_t)i * ms;
    int cnt = n.spikeCount[i], off = n.spikeCountOffset[i];
    for (int k = 0, idx = off; k < cnt; k++, idx++) {
        if (idx >= ms) idx = 0;
        int b1 = (int)((double)h[idx] * (double)n.dt);
        int b2 = (int)((double)h[idx] * (double)n.dt * 100.0);
        if (b1 >= 0 && b1 < n.n_burst_bins) atomicAdd(&n.burstiness[b1], 1.0f);
        if (b2 >= 0 && b2 < n.n_spike_bins) atomicAdd(&n.spikes_hist[b2], 1.0f);
    }
    if (growth && epoch >= 0 && epoch <= n.max_epochs) {
        n.rates_hist[(size_t)epoch * n.N + i] = n.rates[i];
        float r = n.radii[i];
        if (r < n.g_min_radius) r = n.g_min_radius;
        n.radii[i] = r;
        n.radii_hist[(size_t)epoch * n.N + i] = r;
    }
    n.spikeCountOffset[i] = (cnt + off) % ms;
    n.spikeCount[i] = 0;
}

void launch_growth(const NetDev &h, const NetDev *d_net, int epoch, int add_threads, cudaStream_t s)
{
    int nb = (h.N + 255) / 256;
    k_growth_radii<<<nb, 256, 0, s>>>(d_net);
    int sb = 152 * 8;
    k_growth_existing<<<sb, 256, 0, s>>>(d_net);
    k_growth_rmax<<<1, 1024, 0, s>>>(d_net);
    size_t smem = (size_t)((h.N + 31) / 32) * sizeof(uint32_t);
    if (add_threads == 128) k_growth_add<128><<<h.N, 128, smem, s>>>(d_net);
    else if (add_threads == 512) k_growth_add<512><<<h.N, 512, smem, s>>>(d_net);
    else k_growth_add<256><<<h.N, 256, smem, s>>>(d_net);
    k_out_zero<<<nb, 256, 0, s>>>(d_net);
    k_out_count<<<sb, 256, 0, s>>>(d_net);
    k_out_scan<<<1, 1024, 0, s>>>(d_net);
    k_out_fill<<<sb, 256, 0, s>>>(d_net);
    k_record_epoch<<<nb, 256, 0, s>>>(d_net, epoch, true);
}

void launch_record(const NetDev &h, const NetDev *d_net, cudaStream_t s)
{
    k_record_epoch<<<(h.N + 255) / 256, 256, 0, s>>>(d_net, -1, false);
}

// W *= f for every in-use slot (one float multiply each, as a host loop would do it).
__global__ void k_scale_weights(const __grid_constant__ NetDev n, float f)
{
    const size_t S = (size_t)n.Np * (size_t)n.Mq * 4;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < S;
         p += (size_t)gridDim.x * blockDim.x) {
        int k, d;
        pos_slot(p, n.Mq, k, d);
        if (d < n.N && (uint32_t)k < n.count[d]) n.ev[p].W = n.ev[p].W * f;
    }
}

void launch_scale_weights(const NetDev &h, float f, cudaStream_t s)
{
    k_scale_weights<<<152 * 8, 256, 0, s>>>(h, f);
}

void launch_rebuild_maps(const NetDev &h, const NetDev *d_net, cudaStream_t s)
{
    int nb = (h.N + 255) / 256;
    int sb = 152 * 8;
    k_out_zero<<<nb, 256, 0, s>>>(d_net);
    k_out_count<<<sb, 256, 0, s>>>(d_net);
    k_out_scan<<<1, 1024, 0, s>>>(d_net);
    k_out_fill<<<sb, 256, 0, s>>>(d_net);
}

}  // namespace bg3
