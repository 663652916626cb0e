// gbo_sim_forms.inl : the host launchers of one CSG form's simulation kernels.  gbo_sim_tree0.cu, gbo_sim_tree1.cu
// and gbo_sim_tree2.cu each define GBO_SIM_TREE and include this file, so each TREE value's kernels are compiled in
// a translation unit of their own.
#include <atomic>

#include "gbo_sim.cuh"
#include "gbo_wavefront.cuh"

#ifndef GBO_SIM_TREE
#error "GBO_SIM_TREE must name the CSG form (0, 1 or 2)"
#endif

namespace gbo {

template <int TREE, bool PRECISE, bool RCALL>
static void sim_launch_form(const Params& P, const SimLaunch& L)
{
    if (L.kernel_mode != 1) {
        if (P.gen_photon)
            k_simulate_pool<TREE, PRECISE, true, RCALL><<<(unsigned)L.grid, SIM_BLOCK, 0, L.stream>>>(P, L.pool, L.refill,
                                                                                                    L.period);
        else
            k_simulate_pool<TREE, PRECISE, false, RCALL><<<(unsigned)L.grid, SIM_BLOCK, 0, L.stream>>>(P, L.pool, L.refill,
                                                                                                     L.period);
    } else {
        k_simulate<TREE, PRECISE, RCALL><<<(unsigned)((L.n + SIM_BLOCK - 1) / SIM_BLOCK), SIM_BLOCK, 0, L.stream>>>(P);
    }
}

// resident blocks per SM of one kernel, asked of the runtime once per process
template <auto K>
static int resident_blocks()
{
    static std::atomic<int> cached{0};
    int b = cached.load(std::memory_order_relaxed);
    if (b <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, K, SIM_BLOCK, 0) != cudaSuccess || b < 1) b = 1;
        cached.store(b, std::memory_order_relaxed);
    }
    return b;
}

// Kernel mode 3: the start pass, then max_bounce steps of three passes each, all on the launch's stream (the
// passes of a step read their list's length on the device, so the host never waits between them; steps whose list
// is empty return at once).
template <int TREE, bool RCALL, bool PRECISE>
static void wavefront_launch(const Params& P, const SimLaunch& L)
{
    const Wavefront& W = L.wf;
    cudaMemsetAsync(W.count, 0, 2 * (size_t)(P.max_bounce + 1) * sizeof(unsigned long long), L.stream);
    cudaMemsetAsync(W.bins, 0, (size_t)P.max_bounce * WF_CELLS * sizeof(unsigned), L.stream);
    const long long full = (L.n + SIM_BLOCK - 1) / SIM_BLOCK;
    auto grid = [&](int occ) {
        const long long g = (long long)L.sms * occ;
        return (unsigned)(g < full ? g : full);
    };
    k_wf_start<TREE, PRECISE><<<grid(resident_blocks<k_wf_start<TREE, PRECISE>>()), SIM_BLOCK, 0, L.stream>>>(P, W);
    const unsigned g_near = grid(resident_blocks<k_wf_trace<TREE, false, PRECISE>>());
    const unsigned g_walk = grid(resident_blocks<k_wf_trace<TREE, true, PRECISE>>());
    const unsigned g_step = grid(resident_blocks<k_wf_step<TREE, RCALL, PRECISE>>());
    const unsigned g_cells = (unsigned)L.sms * 8u;
    for (int s = 0; s < P.max_bounce; s++) {
        k_wf_trace<TREE, false, PRECISE><<<g_near, SIM_BLOCK, 0, L.stream>>>(P, W, s);
        k_wf_cells_count<TREE><<<g_cells, SIM_BLOCK, 0, L.stream>>>(W, s);
        k_wf_cells_scan<TREE><<<1, WF_SCAN_THREADS, 0, L.stream>>>(W, s);
        k_wf_cells_scatter<TREE><<<g_cells, SIM_BLOCK, 0, L.stream>>>(W, s);
        k_wf_trace<TREE, true, PRECISE><<<g_walk, SIM_BLOCK, 0, L.stream>>>(P, W, s);
        k_wf_step<TREE, RCALL, PRECISE><<<g_step, SIM_BLOCK, 0, L.stream>>>(P, W, s);
    }
}

// The CSG-tree forms always take Philox blocks by call (their code is large enough to miss in the instruction cache
// otherwise); the single-leaf forms inline the rounds unless rng_call asks for the call (binary32 only).
template <int TREE>
void sim_launch(const Params& P, const SimLaunch& L)
{
    // the wavefront form keeps photon indices in 32-bit lists: larger launches run the pool over pregenerated photons
    // instead (and so does a precision-mode launch without accumulator buffers)
    if (L.kernel_mode == 3 && P.gen_photon && L.wf.count && L.n < 0x7fffffffll && (!L.precise || L.wf.acc)) {
        if constexpr (TREE >= 1) {
            if (L.precise) wavefront_launch<TREE, true, true>(P, L);
            else wavefront_launch<TREE, true, false>(P, L);
        } else {
            if (L.precise) wavefront_launch<0, false, true>(P, L);
            else if (L.rng_call) wavefront_launch<0, true, false>(P, L);
            else wavefront_launch<0, false, false>(P, L);
        }
        return;
    }
    if constexpr (TREE >= 1) {
        if (L.precise) sim_launch_form<TREE, true, true>(P, L);
        else sim_launch_form<TREE, false, true>(P, L);
    } else {
        if (L.precise) sim_launch_form<0, true, false>(P, L);
        else if (L.rng_call) sim_launch_form<0, false, true>(P, L);
        else sim_launch_form<0, false, false>(P, L);
    }
}

template <int TREE>
cudaError_t sim_pool_occupancy(bool precise, bool rng_call, int* blocks)
{
    if constexpr (TREE >= 1) {
        if (precise) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_simulate_pool<TREE, true, true, true>,
                                                                          SIM_BLOCK, 0);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_simulate_pool<TREE, false, true, true>, SIM_BLOCK, 0);
    } else {
        if (precise) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_simulate_pool<0, true, true, false>,
                                                                          SIM_BLOCK, 0);
        if (rng_call) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_simulate_pool<0, false, true, true>,
                                                                           SIM_BLOCK, 0);
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k_simulate_pool<0, false, true, false>, SIM_BLOCK, 0);
    }
}

template <int TREE>
void sim_launch_bounded(const Params& P, long long cap, unsigned grid, cudaStream_t s)
{
    k_simulate_bounded<TREE><<<grid, SIM_BLOCK, 0, s>>>(P, cap);
}

template <int TREE>
void trace_rays_launch(bool polish, const Accel& acc, const float3* pos, const float3* dir, int n, float tmin,
                       float tmax, float* t_out, unsigned* boundary_out)
{
    const unsigned g = (unsigned)((n + 127) / 128);
    if (polish) k_trace_rays<TREE, true><<<g, 128>>>(acc, pos, dir, n, tmin, tmax, t_out, boundary_out);
    else k_trace_rays<TREE, false><<<g, 128>>>(acc, pos, dir, n, tmin, tmax, t_out, boundary_out);
}

GBO_SIM_FORM_INSTANCES(, GBO_SIM_TREE)

}  // namespace gbo
