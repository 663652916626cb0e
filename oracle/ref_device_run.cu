/*
 * ref_device_run.cu : host driver of the reference-header device build (TEST INFRASTRUCTURE ONLY).
 *
 * Built by `make -C oracle ref-device-run` into oracle/_ref/libref_device_run.so on the machine with the GPU (it
 * contains no reference code).  It loads oracle/_ref/ref_device.cubin (compiled from the reference's headers where
 * the reference tree is, see ref_device.cu) through the CUDA driver API, uploads one event's inputs described by
 * the oracle's orc_sim struct, creates the boundary and scintillation textures with the reference's descriptors
 * (linear filter, normalized coordinates, wrap: qudarap/QTex.cc:255-275) and launches ref_simulate_kernel with one
 * thread per photon.  Photons and flag histories come back to host memory.
 *
 * Called from tests/golden/make_device_golden.py, which writes the reference-device fixtures.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

extern "C" {
#include "oracle.h"
}
#include "ref_device.h"

namespace {

char g_err[512];

#define RCU(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    snprintf(g_err, sizeof g_err, "%s: %s", #x, cudaGetErrorString(e_)); goto fail; } } while (0)
#define RDR(x) do { CUresult r_ = (x); if (r_ != CUDA_SUCCESS) { const char* s_ = nullptr; cuGetErrorString(r_, &s_); \
    snprintf(g_err, sizeof g_err, "%s: %s", #x, s_ ? s_ : "?"); goto fail; } } while (0)

cudaError_t make_tex(const float* data, int nx, int ny, bool f4, cudaArray_t* arr, cudaTextureObject_t* tex)
{
    cudaChannelFormatDesc ch = f4 ? cudaCreateChannelDesc<float4>() : cudaCreateChannelDesc<float>();
    cudaError_t e = cudaMallocArray(arr, &ch, (size_t)nx, (size_t)ny);
    if (e != cudaSuccess) return e;
    size_t row = (size_t)nx * (f4 ? 16 : 4);
    e = cudaMemcpy2DToArray(*arr, 0, 0, data, row, row, (size_t)ny, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof rd);
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = *arr;
    cudaTextureDesc td;
    memset(&td, 0, sizeof td);
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    return cudaCreateTextureObject(tex, &rd, &td, nullptr);
}

template <typename T>
cudaError_t upload(const void* src, size_t bytes, T** dst)
{
    size_t n = bytes ? bytes : 16;
    cudaError_t e = cudaMalloc((void**)dst, n);
    if (e != cudaSuccess) return e;
    if (bytes) return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    return cudaMemset(*dst, 0, n);
}

/* world box of every instance from its solid's prim boxes (CSGPrim q2.xyzw, q3.xy) through the forward transform
   (row-vector convention: world = local x M, translation in q3), padded generously: a prefilter only */
void instance_boxes(const orc_sim* s, std::vector<float>& box)
{
    const orc_geom& g = s->geom;
    box.assign((size_t)g.num_inst * 6, 0.f);
    for (int i = 0; i < g.num_inst; i++) {
        const gbo_qat4& m = g.inst[i];
        int gas = m.q1.i[3];
        const gbo_csgsolid& so = g.solid[gas];
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int k = 0; k < so.numPrim; k++) {
            const gbo_csgprim& pr = g.prim[so.primOffset + k];
            double mn[3] = {pr.q2.f[0], pr.q2.f[1], pr.q2.f[2]};
            double mx[3] = {pr.q2.f[3], pr.q3.f[0], pr.q3.f[1]};
            for (int c = 0; c < 8; c++) {
                double p[3] = {(c & 1) ? mx[0] : mn[0], (c & 2) ? mx[1] : mn[1], (c & 4) ? mx[2] : mn[2]};
                for (int a = 0; a < 3; a++) {
                    double w = p[0] * m.q0.f[a] + p[1] * m.q1.f[a] + p[2] * m.q2.f[a] + m.q3.f[a];
                    lo[a] = w < lo[a] ? w : lo[a];
                    hi[a] = w > hi[a] ? w : hi[a];
                }
            }
        }
        double ext = 0.0;
        for (int a = 0; a < 3; a++) ext = fmax(ext, fmax(fabs(lo[a]), fabs(hi[a])));
        double pad = 1.0 + 1e-4 * ext;
        for (int a = 0; a < 3; a++) {
            box[6 * i + a] = (float)(lo[a] - pad);
            box[6 * i + 3 + a] = (float)(hi[a] + pad);
        }
    }
}

}  // namespace

extern "C" const char* ref_device_last_error(void) { return g_err; }

/* Run one launch of the reference-header device build.  sizes = {num_node, num_prim, num_solid, num_itra,
 * num_plan, num_optical_rows}.  input_photon (num_photon records, or NULL) seeds the photon buffer, as the
 * reference's evt->photon holds the input photons that INPUT_PHOTON gensteps read.  Returns 0 on success. */
extern "C" int ref_device_simulate(const char* cubin_path, const orc_sim* s, const int32_t* sizes,
                                   const gbo_quad6* gs, int64_t num_gs, const int32_t* seed_idx,
                                   const gbo_sphoton* input_photon, uint64_t photon_offset, int32_t event_index,
                                   int64_t num_photon, gbo_sphoton* photon_out, gbo_seq* seq_out, float* kernel_ms)
{
    g_err[0] = 0;
    int rc = 1;
    CUmodule mod = nullptr;
    CUfunction fn = nullptr;
    cudaArray_t bnd_arr = nullptr, icdf_arr = nullptr;
    cudaTextureObject_t bnd_tex = 0, icdf_tex = 0;
    void *d_node = nullptr, *d_prim = nullptr, *d_solid = nullptr, *d_inst = nullptr, *d_inst_inv = nullptr,
         *d_itra = nullptr, *d_plan = nullptr, *d_optical = nullptr, *d_box = nullptr, *d_gs = nullptr,
         *d_seed = nullptr, *d_photon = nullptr, *d_seq = nullptr;
    std::vector<float> box;
    ref_dev_params P;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int block = 128;
    unsigned grid = (unsigned)((num_photon + block - 1) / block);
    void* args[1] = {&P};
    memset(&P, 0, sizeof P);
    instance_boxes(s, box);

    RCU(cudaFree(0));
    RDR(cuModuleLoad(&mod, cubin_path));
    RDR(cuModuleGetFunction(&fn, mod, "ref_simulate_kernel"));
    RDR(cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, 0));
    RCU(cudaDeviceSetLimit(cudaLimitStackSize, 4096));

    RCU(upload(s->geom.node, (size_t)sizes[0] * 64, &d_node));
    RCU(upload(s->geom.prim, (size_t)sizes[1] * 64, &d_prim));
    RCU(upload(s->geom.solid, (size_t)sizes[2] * 48, &d_solid));
    RCU(upload(s->geom.inst, (size_t)s->geom.num_inst * 64, &d_inst));
    RCU(upload(s->geom.inst_inv, (size_t)s->geom.num_inst * 64, &d_inst_inv));
    RCU(upload(s->geom.itra, (size_t)sizes[3] * 64, &d_itra));
    RCU(upload(s->geom.plan, (size_t)sizes[4] * 16, &d_plan));
    RCU(upload(s->optical, (size_t)sizes[5] * 16, &d_optical));
    RCU(upload(box.data(), box.size() * 4, &d_box));
    RCU(upload(gs, (size_t)num_gs * 96, &d_gs));
    RCU(upload(seed_idx, (size_t)num_photon * 4, &d_seed));
    RCU(upload(input_photon, input_photon ? (size_t)num_photon * 64 : 0, &d_photon));
    if (!input_photon && num_photon) {
        RCU(cudaFree(d_photon));
        d_photon = nullptr;
        RCU(cudaMalloc(&d_photon, (size_t)num_photon * 64));
        RCU(cudaMemset(d_photon, 0, (size_t)num_photon * 64));
    }
    RCU(cudaMalloc(&d_seq, (size_t)(num_photon ? num_photon : 1) * 32));
    RCU(cudaMemset(d_seq, 0, (size_t)(num_photon ? num_photon : 1) * 32));
    RCU(make_tex(s->bnd.data, s->bnd.nx, s->bnd.ny, true, &bnd_arr, &bnd_tex));
    RCU(make_tex(s->icdf.data, s->icdf.nx, s->icdf.ny, false, &icdf_arr, &icdf_tex));

    P.node = d_node; P.prim = d_prim; P.solid = d_solid; P.inst = d_inst; P.inst_inv = d_inst_inv;
    P.inst_box = (const float*)d_box; P.itra = d_itra; P.plan = d_plan; P.num_inst = s->geom.num_inst;
    P.bnd_tex = (uint64_t)bnd_tex; P.bnd_nx = (uint32_t)s->bnd.nx; P.bnd_ny = (uint32_t)s->bnd.ny;
    P.bnd_nm0 = s->bnd_nm0; P.bnd_nms = s->bnd_nms; P.optical = (const uint32_t*)d_optical;
    P.icdf_tex = (uint64_t)icdf_tex; P.hd_factor = s->hd_factor;
    P.max_bounce = s->max_bounce; P.max_time = s->max_time; P.tmin = s->tmin; P.tmin0 = s->tmin0; P.tmax = s->tmax;
    P.eps0_mask = s->eps0_mask; P.seed = s->seed; P.offset = s->offset;
    P.skipahead_event_offset = s->skipahead_event_offset;
    P.genstep = d_gs; P.seed_idx = (const int32_t*)d_seed; P.photon_offset = photon_offset;
    P.event_index = event_index; P.num_photon = num_photon; P.photon = d_photon; P.seq = d_seq;

    RCU(cudaEventCreate(&e0));
    RCU(cudaEventCreate(&e1));
    RCU(cudaEventRecord(e0, 0));
    if (grid) RDR(cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, 0, args, nullptr));
    RCU(cudaEventRecord(e1, 0));
    RCU(cudaDeviceSynchronize());
    if (kernel_ms) RCU(cudaEventElapsedTime(kernel_ms, e0, e1));
    if (num_photon) {
        RCU(cudaMemcpy(photon_out, d_photon, (size_t)num_photon * 64, cudaMemcpyDeviceToHost));
        if (seq_out) RCU(cudaMemcpy(seq_out, d_seq, (size_t)num_photon * 32, cudaMemcpyDeviceToHost));
    }
    rc = 0;
fail:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (bnd_tex) cudaDestroyTextureObject(bnd_tex);
    if (icdf_tex) cudaDestroyTextureObject(icdf_tex);
    if (bnd_arr) cudaFreeArray(bnd_arr);
    if (icdf_arr) cudaFreeArray(icdf_arr);
    for (void* p : {d_node, d_prim, d_solid, d_inst, d_inst_inv, d_itra, d_plan, d_optical, d_box, d_gs, d_seed,
                    d_photon, d_seq})
        if (p) cudaFree(p);
    if (mod) cuModuleUnload(mod);
    return rc;
}
