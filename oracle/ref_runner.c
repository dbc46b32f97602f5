/*
 * ref_runner.c -- host driver for the reference's own CUDA kernels (TEST
 * INFRASTRUCTURE ONLY: it produces the golden outputs that pin the CPU oracle).
 *
 * oracle/ref_build.py compiles the reference's five unmodified CUDA translation units to
 * cubins; this file loads them with the CUDA driver API and launches the kernels in
 * the order, shapes and arguments of the reference's host code:
 *   construction   FastReg ctor (src/fastreg/fastreg.cpp:24-46), Solver ctor
 *                  (src/fastreg/solver.cpp:7-65), field ctors (vector_fields.cpp,
 *                  scalar_fields.cpp, volume.cpp): clears, identity psi/psi_inv, rho_0
 *   operator()     four Volume::initialise (fastreg.cpp:58-63), estimate_psi
 *                  (src/fastreg/cuda/solver.cu:295-444) at verbosity 0, and the
 *                  float2 -> (float, short) split of get_image_data (fastreg.cpp:3-22)
 * The reference's five streams are replaced by one stream: its legacy-default-stream
 * launches and the per-iteration host syncs already serialise every dependency
 * (solver.cu:375-407).  One deviation for determinism: the `updates` buffer, whose
 * boundary entries the reference leaves as uninitialised cudaMalloc memory
 * (reductor.cpp:23), is zeroed once.
 *
 * Kernel arguments are the reference's device views, all {T *data; int3 dims}
 * (include/cuda/{volume,vector_fields,scalar_fields}.hpp), i.e. 24-byte structs.
 */
#include <cuda.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    CUdeviceptr data;
    int dims[3];
    int pad_;
} rr_view;

enum { M_SOLVER, M_VF, M_REDUCTOR, M_SF, M_VOLUME, M_COUNT };
static const char *MOD_FILES[M_COUNT] = {"solver.cubin", "vector_fields.cubin", "reductor.cubin", "scalar_fields.cubin",
                                         "volume.cubin"};

static char g_err[512];
const char *rr_last_error(void) { return g_err; }

#define CK(call)                                                                               \
    do {                                                                                       \
        CUresult r_ = (call);                                                                  \
        if (r_ != CUDA_SUCCESS) {                                                              \
            const char *s_ = NULL;                                                             \
            cuGetErrorString(r_, &s_);                                                         \
            snprintf(g_err, sizeof g_err, "%s failed: %s (line %d)", #call, s_ ? s_ : "?", __LINE__); \
            goto fail;                                                                         \
        }                                                                                      \
    } while (0)

/* Find the kernel of `mod` whose mangled name holds `<len><name>` followed by `next`
 * ('E' for plain kernels, 'I' for template instances) and, if given, `extra`. */
static int find_fn(CUmodule mod, const char *name, char next, const char *extra, CUfunction *out) {
    unsigned n = 0;
    if (cuModuleGetFunctionCount(&n, mod) != CUDA_SUCCESS || n == 0) return -1;
    CUfunction *fs = (CUfunction *)malloc(sizeof(CUfunction) * n);
    if (cuModuleEnumerateFunctions(fs, n, mod) != CUDA_SUCCESS) {
        free(fs);
        return -1;
    }
    char key[160];
    snprintf(key, sizeof key, "%d%s%c", (int)strlen(name), name, next);
    int found = -1;
    for (unsigned k = 0; k < n; ++k) {
        const char *nm = NULL;
        if (cuFuncGetName(&nm, fs[k]) != CUDA_SUCCESS || !nm) continue;
        if (strstr(nm, key) && (!extra || strstr(nm, extra))) {
            *out = fs[k];
            found = 0;
            break;
        }
    }
    free(fs);
    if (found) snprintf(g_err, sizeof g_err, "kernel %s%s not found", key, extra ? extra : "");
    return found;
}

static int div_up(int a, int b) { return (a + b - 1) / b; }

static CUresult launch2d(CUfunction f, int X, int Y, int bx, int by, CUstream s, void **args) {
    return cuLaunchKernel(f, div_up(X, bx), div_up(Y, by), 1, bx, by, 1, 0, s, args, NULL);
}

typedef struct {
    int max_iter;
    int reset_iter;
    float max_update_norm, rho_0, tau, w_reg, alpha, p, C;
} rr_params;

/* Runs one registration with the reference kernels.  Host arrays: T/S float[N],
 * labels short[N]; outputs as for FastReg::operator(); psi/psi_inv 3 planes of N;
 * trace_norm/trace_idx hold one entry per iteration; ms_out (may be NULL) receives the
 * device-event time of FastReg::operator() from the input upload to the last apply
 * ([0]) and of estimate_psi alone ([1]).  Returns iterations run, or -1. */
int rr_register(const char *cubin_dir, const int *dims, const rr_params *P, const float *T, const short *labT,
                const float *S, const short *labS, float *out_T, short *out_labT, float *out_S, short *out_labS,
                float *psi_out, float *psi_inv_out, float *trace_norm, long long *trace_idx, float *ms_out) {
    CUmodule mods[M_COUNT] = {0};
    CUdeviceptr bufs[32];
    int nbufs = 0;
    CUstream st = 0;
    CUcontext ctx = 0;
    CUdevice dev = 0;
    int ran = -1;
    const int X = dims[0], Y = dims[1], Z = dims[2];
    const size_t N = (size_t)X * Y * Z;
    float *h_f2 = NULL, *h_f4 = NULL;

    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    for (int m = 0; m < M_COUNT; ++m) {
        char path[1024];
        snprintf(path, sizeof path, "%s/%s", cubin_dir, MOD_FILES[m]);
        CK(cuModuleLoad(&mods[m], path));
    }
    CK(cuStreamCreate(&st, CU_STREAM_NON_BLOCKING));

    CUfunction k_vol_clear, k_vol_init, k_vf_clear, k_identity, k_apply, k_grad, k_interp_L, k_lap, k_lap_v, k_dvv,
        k_jac_clear, k_jac, k_sf_clear, k_density, k_potential, k_div, k_upd_rho, k_upd_v, k_upd_psi, k_upd_psi_inv,
        k_max;
    if (find_fn(mods[M_VOLUME], "clear_kernel", 'E', NULL, &k_vol_clear) ||
        find_fn(mods[M_VOLUME], "initialise_kernel", 'E', NULL, &k_vol_init) ||
        find_fn(mods[M_VF], "clear_kernel", 'E', NULL, &k_vf_clear) ||
        find_fn(mods[M_VF], "init_identity_kernel", 'E', NULL, &k_identity) ||
        find_fn(mods[M_VF], "apply_kernel", 'E', NULL, &k_apply) ||
        find_fn(mods[M_VF], "estimate_gradient_kernel", 'E', NULL, &k_grad) ||
        find_fn(mods[M_VF], "interpolate_laplacian_kernel", 'E', NULL, &k_interp_L) ||
        find_fn(mods[M_VF], "estimate_laplacian_kernel", 'E', NULL, &k_lap) ||
        find_fn(mods[M_VF], "estimate_laplacian_velocity_kernel", 'E', NULL, &k_lap_v) ||
        find_fn(mods[M_VF], "calc_dv_v_kernel", 'E', NULL, &k_dvv) ||
        find_fn(mods[M_VF], "clear_jacobian_kernel", 'E', NULL, &k_jac_clear) ||
        find_fn(mods[M_VF], "estimate_jacobian_kernel", 'E', NULL, &k_jac) ||
        find_fn(mods[M_SF], "clear_kernel", 'E', NULL, &k_sf_clear) ||
        find_fn(mods[M_SF], "init_density_kernel", 'E', NULL, &k_density) ||
        find_fn(mods[M_SOLVER], "calculate_potential_gradient_kernel", 'E', NULL, &k_potential) ||
        find_fn(mods[M_SOLVER], "calc_divergence_kernel", 'E', NULL, &k_div) ||
        find_fn(mods[M_SOLVER], "update_density_kernel", 'E', NULL, &k_upd_rho) ||
        find_fn(mods[M_SOLVER], "update_velocity_kernel", 'E', NULL, &k_upd_v) ||
        find_fn(mods[M_SOLVER], "update_psi_kernel", 'E', NULL, &k_upd_psi) ||
        find_fn(mods[M_SOLVER], "update_psi_inv_kernel", 'E', NULL, &k_upd_psi_inv))
        goto fail;

    /* reduction launch shape: get_num_blocks_and_threads(n, 65536, 512) (precomp.cpp:28-51) */
    int threads = (N < 1024) ? 1 : 512;
    if (N < 1024) {
        unsigned v = (unsigned)((N + 1) / 2);
        v--; v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16; v++;
        threads = (int)v;
    }
    int blocks = (int)((N + (size_t)threads * 2 - 1) / ((size_t)threads * 2));
    if (blocks > 65536) blocks = 65536;
    const int pow2 = (N & (N - 1)) == 0;
    char tmpl[64];
    snprintf(tmpl, sizeof tmpl, "ILj%dELb%dE", threads, pow2);
    if (find_fn(mods[M_REDUCTOR], "reduce_max_kernel", 'I', tmpl, &k_max)) goto fail;

    /* Device memory.  Every buffer gets a zeroed tail of (X*Y + X + 64) float4s: the
     * reference's unchecked corner reads (Volume/VectorField operator(), used by
     * interpolate_intensity and interpolate_field) reach up to X*Y + X + 1 elements
     * past the last voxel, with weight 0; the tail keeps those reads inside the
     * allocation. */
    const size_t tail = ((size_t)X * Y + X + 64) * 16;
#define ALLOC(var, bytes)                               \
    CUdeviceptr var;                                    \
    CK(cuMemAlloc(&var, (bytes) + tail));               \
    bufs[nbufs++] = var;                                \
    CK(cuMemsetD8(var, 0, (bytes) + tail));
    ALLOC(d_phi_global, N * 8);
    ALLOC(d_phi_global_psi_inv, N * 8);
    ALLOC(d_phi_n, N * 8);
    ALLOC(d_phi_n_psi, N * 8);
    ALLOC(d_psi, N * 16);
    ALLOC(d_psi_inv, N * 16);
    ALLOC(d_v, N * 16);
    ALLOC(d_rho, N * 4);
    ALLOC(d_div, N * 4);
    ALLOC(d_nabla_phi_n, N * 16);
    ALLOC(d_J_inv, N * 64);
    ALLOC(d_L, N * 16);
    ALLOC(d_L_o_psi_inv, N * 16);
    ALLOC(d_dv_v, N * 16);
    ALLOC(d_delta_v, N * 16);
    ALLOC(d_nabla_U, N * 16);
    ALLOC(d_updates, N * 16);
    ALLOC(d_max_out, (size_t)blocks * 8);
    ALLOC(d_img_T, N * 4);
    ALLOC(d_lab_T, N * 2);
    ALLOC(d_img_S, N * 4);
    ALLOC(d_lab_S, N * 2);
#undef ALLOC

    rr_view vg = {d_phi_global, {X, Y, Z}, 0}, vgw = {d_phi_global_psi_inv, {X, Y, Z}, 0};
    rr_view vn = {d_phi_n, {X, Y, Z}, 0}, vnw = {d_phi_n_psi, {X, Y, Z}, 0};
    rr_view fpsi = {d_psi, {X, Y, Z}, 0}, fpsi_inv = {d_psi_inv, {X, Y, Z}, 0}, fv = {d_v, {X, Y, Z}, 0};
    rr_view srho = {d_rho, {X, Y, Z}, 0}, sdiv = {d_div, {X, Y, Z}, 0};
    rr_view fgrad = {d_nabla_phi_n, {X, Y, Z}, 0}, jinv = {d_J_inv, {X, Y, Z}, 0}, fL = {d_L, {X, Y, Z}, 0};
    rr_view fLo = {d_L_o_psi_inv, {X, Y, Z}, 0}, fdvv = {d_dv_v, {X, Y, Z}, 0}, fdv = {d_delta_v, {X, Y, Z}, 0};
    rr_view fU = {d_nabla_U, {X, Y, Z}, 0};

    /* ---- construction ---- */
    {
        void *a1[] = {&vg};
        CK(launch2d(k_vol_clear, X, Y, 64, 16, st, a1));
        void *a2[] = {&vgw};
        CK(launch2d(k_vol_clear, X, Y, 64, 16, st, a2));
        void *a3[] = {&vn};
        CK(launch2d(k_vol_clear, X, Y, 64, 16, st, a3));
        void *a4[] = {&vnw};
        CK(launch2d(k_vol_clear, X, Y, 64, 16, st, a4));
        rr_view *vfs[] = {&fpsi, &fpsi_inv, &fv, &fgrad, &fL, &fLo, &fdvv, &fdv, &fU};
        for (int k = 0; k < 9; ++k) {
            void *a[] = {vfs[k]};
            CK(launch2d(k_vf_clear, X, Y, 64, 16, st, a));
        }
        void *ai[] = {&fpsi};
        CK(launch2d(k_identity, X, Y, 64, 16, st, ai));
        void *aj[] = {&fpsi_inv};
        CK(launch2d(k_identity, X, Y, 64, 16, st, aj));
        void *ar[] = {&srho};
        CK(launch2d(k_sf_clear, X, Y, 64, 16, st, ar));
        float rho0 = P->rho_0;
        void *ad[] = {&srho, &rho0};
        CK(launch2d(k_density, X, Y, 64, 16, st, ad));
        void *av[] = {&sdiv};
        CK(launch2d(k_sf_clear, X, Y, 64, 16, st, av));
        void *aJ[] = {&jinv};
        CK(launch2d(k_jac_clear, X, Y, 64, 16, st, aJ));
        CK(cuMemsetD8Async(d_updates, 0, N * 16, st));
    }

    /* ---- FastReg::operator(): pack the inputs ---- */
    CUevent ev[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) CK(cuEventCreate(&ev[k], CU_EVENT_DEFAULT));
    CK(cuStreamSynchronize(st));
    CK(cuEventRecord(ev[0], st));
    CK(cuMemcpyHtoD(d_img_T, T, N * 4));
    CK(cuMemcpyHtoD(d_lab_T, labT, N * 2));
    CK(cuMemcpyHtoD(d_img_S, S, N * 4));
    CK(cuMemcpyHtoD(d_lab_S, labS, N * 2));
    {
        void *a1[] = {&vg, &d_img_T, &d_lab_T};
        CK(launch2d(k_vol_init, X, Y, 64, 16, st, a1));
        void *a2[] = {&vgw, &d_img_T, &d_lab_T};
        CK(launch2d(k_vol_init, X, Y, 64, 16, st, a2));
        void *a3[] = {&vn, &d_img_S, &d_lab_S};
        CK(launch2d(k_vol_init, X, Y, 64, 16, st, a3));
        void *a4[] = {&vnw, &d_img_S, &d_lab_S};
        CK(launch2d(k_vol_init, X, Y, 64, 16, st, a4));
    }

    /* ---- estimate_psi ---- */
    CK(cuEventRecord(ev[1], st));
    {
        void *ag[] = {&vn, &fgrad}; /* VolumeDifferentiator{phi_n} */
        CK(launch2d(k_grad, X, Y, 64, 16, st, ag));
        float rho0 = P->rho_0;
        void *ad[] = {&srho, &rho0};
        CK(launch2d(k_density, X, Y, 32, 16, st, ad));
    }
    h_f2 = (float *)malloc((size_t)blocks * 8);
    float alpha = P->alpha, t = P->alpha, w_reg = P->w_reg, tau = P->tau, pp = P->p, CC = P->C;
    int dx = X, dy = Y, dz = Z;
    unsigned n_u = (unsigned)N;
    int iter = 1;
    ran = 0;
    while (iter <= P->max_iter) {
        void *a_div[] = {&d_rho, &d_v, &d_div, &dx, &dy, &dz};
        CK(launch2d(k_div, X, Y, 32, 16, st, a_div));
        void *a_urho[] = {&d_rho, &d_div, &alpha, &dx, &dy, &dz};
        CK(launch2d(k_upd_rho, X, Y, 32, 16, st, a_urho));
        void *a_jac[] = {&fpsi_inv, &jinv}; /* Differentiator{psi_inv} */
        CK(launch2d(k_jac, X, Y, 32, 16, st, a_jac));
        void *a_lap[] = {&fpsi, &fL}; /* SecondOrderDifferentiator{psi} */
        CK(launch2d(k_lap, X, Y, 32, 16, st, a_lap));
        void *a_il[] = {&fL, &fLo, &fpsi_inv};
        CK(launch2d(k_interp_L, X, Y, 32, 16, st, a_il));
        void *a_pot[] = {&d_phi_n, &d_phi_global_psi_inv, &d_nabla_phi_n, &d_J_inv, &d_L_o_psi_inv, &d_nabla_U,
                         &w_reg, &dx, &dy, &dz};
        CK(launch2d(k_potential, X, Y, 64, 16, st, a_pot));
        void *a_dvv[] = {&fv, &fdvv};
        CK(launch2d(k_dvv, X, Y, 32, 16, st, a_dvv));
        void *a_lv[] = {&fv, &fdv}; /* SecondOrderDifferentiator{v} */
        CK(launch2d(k_lap_v, X, Y, 32, 16, st, a_lv));
        void *a_uv[] = {&d_v, &d_dv_v, &d_delta_v, &d_rho, &d_nabla_U, &alpha, &t, &tau, &pp, &CC, &dx, &dy, &dz};
        CK(launch2d(k_upd_v, X, Y, 64, 16, st, a_uv));
        void *a_up[] = {&d_psi, &d_v, &d_updates, &alpha, &dx, &dy, &dz};
        CK(launch2d(k_upd_psi, X, Y, 32, 16, st, a_up));
        void *a_upi[] = {&d_psi_inv, &d_J_inv, &d_v, &alpha, &dx, &dy, &dz};
        CK(launch2d(k_upd_psi_inv, X, Y, 32, 16, st, a_upi));
        void *a_ap[] = {&vg, &vgw, &fpsi_inv};
        CK(launch2d(k_apply, X, Y, 32, 16, st, a_ap));
        /* max update norm: reduce_max + host finish (reductor.cpp:74-80,107-120) */
        void *a_max[] = {&d_updates, &d_max_out, &n_u};
        CK(cuLaunchKernel(k_max, blocks, 1, 1, threads, 1, 1, (unsigned)(threads * 8), st, a_max, NULL));
        CK(cuStreamSynchronize(st));
        CK(cuMemcpyDtoH(h_f2, d_max_out, (size_t)blocks * 8));
        float best = 0.f, best_i = 0.f;
        for (int b = 0; b < blocks; ++b)
            if (h_f2[2 * b] > best) {
                best = h_f2[2 * b];
                best_i = h_f2[2 * b + 1];
            }
        trace_norm[iter - 1] = best;
        trace_idx[iter - 1] = (long long)best_i;
        ran = iter;
        if (best <= P->max_update_norm) break;
        if (iter == P->max_iter) break;
        iter++;
        t += alpha;
        if (P->reset_iter > 0 && iter % P->reset_iter == 0) t = P->alpha;
    }
    {
        void *a_ap[] = {&vn, &vnw, &fpsi};
        CK(launch2d(k_apply, X, Y, 32, 16, st, a_ap));
    }
    CK(cuEventRecord(ev[2], st));
    CK(cuStreamSynchronize(st));
    if (ms_out) {
        CK(cuEventElapsedTime(&ms_out[0], ev[0], ev[2]));
        CK(cuEventElapsedTime(&ms_out[1], ev[1], ev[2]));
    }
    for (int k = 0; k < 3; ++k) cuEventDestroy(ev[k]);

    /* ---- get_image_data: float2 -> float + (short) label ---- */
    free(h_f2);
    h_f2 = (float *)malloc(N * 8);
    CK(cuMemcpyDtoH(h_f2, d_phi_global_psi_inv, N * 8));
    for (size_t i = 0; i < N; ++i) {
        out_T[i] = h_f2[2 * i];
        out_labT[i] = (short)h_f2[2 * i + 1];
    }
    CK(cuMemcpyDtoH(h_f2, d_phi_n_psi, N * 8));
    for (size_t i = 0; i < N; ++i) {
        out_S[i] = h_f2[2 * i];
        out_labS[i] = (short)h_f2[2 * i + 1];
    }
    h_f4 = (float *)malloc(N * 16);
    CK(cuMemcpyDtoH(h_f4, d_psi, N * 16));
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) psi_out[c * N + i] = h_f4[4 * i + c];
    CK(cuMemcpyDtoH(h_f4, d_psi_inv, N * 16));
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) psi_inv_out[c * N + i] = h_f4[4 * i + c];

    goto done;
fail:
    ran = -1;
done:
    free(h_f2);
    free(h_f4);
    for (int k = 0; k < nbufs; ++k) cuMemFree(bufs[k]);
    if (st) cuStreamDestroy(st);
    for (int m = 0; m < M_COUNT; ++m)
        if (mods[m]) cuModuleUnload(mods[m]);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return ran;
}

/* The reference's two field kernels that its registration never calls
 * (src/fastreg/cuda/vector_fields.cu:109-136,194-225), run as its host code would:
 *   op 0  estimate_inverse (vector_fields.cu:125-136): `sweeps` launches (48 in the
 *         reference) of estimate_inverse_kernel(psi, psi_inv), psi_inv updated in place;
 *         a is psi, b the initial psi_inv, out the final psi_inv;
 *   op 1  interpolate_gradient (vector_fields.cu:217-225): interpolate_gradient_kernel(
 *         field, out, psi); a is psi, b the field, out = field o psi.
 * Host arrays are 3 planes of N floats (packed to and from float4 with w = 0); every
 * buffer has the zeroed tail described in rr_register.  Returns 0, or -1. */
int rr_field_op(const char *cubin_dir, const int *dims, int op, int sweeps, const float *a, const float *b,
                float *out) {
    CUmodule mod = 0;
    CUdeviceptr bufs[3] = {0, 0, 0};
    CUstream st = 0;
    CUcontext ctx = 0;
    CUdevice dev = 0;
    int rc = -1;
    const int X = dims[0], Y = dims[1], Z = dims[2];
    const size_t N = (size_t)X * Y * Z;
    const size_t tail = ((size_t)X * Y + X + 64) * 16;
    float *h = (float *)calloc(N * 4, sizeof(float));
    if (!h) {
        snprintf(g_err, sizeof g_err, "out of host memory");
        return -1;
    }
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    {
        char path[1024];
        snprintf(path, sizeof path, "%s/%s", cubin_dir, MOD_FILES[M_VF]);
        CK(cuModuleLoad(&mod, path));
    }
    CK(cuStreamCreate(&st, CU_STREAM_NON_BLOCKING));
    CUfunction k;
    if (find_fn(mod, op == 0 ? "estimate_inverse_kernel" : "interpolate_gradient_kernel", 'E', NULL, &k)) goto fail;
    for (int j = 0; j < 3; ++j) {
        CK(cuMemAlloc(&bufs[j], N * 16 + tail));
        CK(cuMemsetD8(bufs[j], 0, N * 16 + tail));
    }
    const float *src[2] = {a, b};
    for (int j = 0; j < 2; ++j) {
        for (size_t i = 0; i < N; ++i)
            for (int c = 0; c < 3; ++c) h[4 * i + c] = src[j][c * N + i];
        CK(cuMemcpyHtoD(bufs[j], h, N * 16));
    }
    rr_view va = {bufs[0], {X, Y, Z}, 0}, vb = {bufs[1], {X, Y, Z}, 0}, vo = {bufs[2], {X, Y, Z}, 0};
    CUdeviceptr result = bufs[2];
    if (op == 0) {
        void *args[] = {&va, &vb};
        for (int s = 0; s < sweeps; ++s) {
            CK(launch2d(k, X, Y, 64, 16, st, args));
            CK(cuStreamSynchronize(st));
        }
        result = bufs[1];
    } else {
        void *args[] = {&vb, &vo, &va};
        CK(launch2d(k, X, Y, 64, 16, st, args));
    }
    CK(cuStreamSynchronize(st));
    CK(cuMemcpyDtoH(h, result, N * 16));
    for (size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) out[c * N + i] = h[4 * i + c];
    rc = 0;
    goto done;
fail:
    rc = -1;
done:
    free(h);
    for (int j = 0; j < 3; ++j)
        if (bufs[j]) cuMemFree(bufs[j]);
    if (st) cuStreamDestroy(st);
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return rc;
}
