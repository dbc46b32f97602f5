/*
 * fr_oracle.c -- CPU oracle for the fastreg registration loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it; the product library
 * (fastreg_gb300/csrc) never links, calls or falls back to it.
 *
 * It restates, voxel by voxel, the arithmetic of fastreg's registration loop
 * (src/fastreg/cuda/solver.cu:295-444 and the kernels it launches) in plain C.
 * The same source is compiled twice:
 *   - FRO_REAL=float  (symbols fro32_*): op-order matched to the CUDA kernels
 *     of this repository, so GPU and oracle agree bit for bit;
 *   - FRO_REAL=double (symbols fro64_*): the FP64 accuracy reference.
 *
 * Op-order contract shared with the kernels (fr_ref.cuh, fr_sob.cuh):
 *   - no contraction of a*b+c anywhere (the kernels build with --fmad=false,
 *     this file with -ffp-contract=off); the only fused multiply-adds are the
 *     explicit ones inside lerp, as in include/cuda/cuda_utils.hpp:43-46;
 *   - sums are evaluated left to right exactly as written in the reference;
 *   - x/2 is evaluated as x*0.5 (the reference's __fdividef(x, 2.f) on a
 *     power of two), other divisions are IEEE divisions;
 *   - the update norm is sqrt rounded toward -inf (reference __fsqrt_rd,
 *     include/cuda/cuda_utils.hpp:251-253).
 *
 * Layouts: scalar fields are X*Y*Z floats, x fastest (idx = x + X*(y + Y*z),
 * include/cuda/device.hpp:17-19); vector fields are three such planes
 * back to back (component c at offset c*N).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef FRO_REAL
#define FRO_REAL float
#endif

#define FRO_IS_FLOAT (sizeof(FRO_REAL) == 4)

typedef FRO_REAL real;

#if defined(FRO_DOUBLE)
#define FN(name) fro64_##name
#define FMA_ fma
#define FMIN_ fmin
#define FMAX_ fmax
#define FLOOR_ floor
#define FABS_ fabs
#else
#define FN(name) fro32_##name
#define FMA_ fmaf
#define FMIN_ fminf
#define FMAX_ fmaxf
#define FLOOR_ floorf
#define FABS_ fabsf
#endif

#define R(x) ((real)(x))

typedef struct {
    int X, Y, Z;
} fro_dims;

static inline int64_t nvox(const fro_dims *d) { return (int64_t)d->X * d->Y * d->Z; }

static inline int64_t lin(const fro_dims *d, int x, int y, int z) {
    return (int64_t)x + (int64_t)d->X * ((int64_t)y + (int64_t)d->Y * z);
}

static inline int is_interior(const fro_dims *d, int x, int y, int z) {
    return x >= 1 && x <= d->X - 2 && y >= 1 && y <= d->Y - 2 && z >= 1 && z <= d->Z - 2;
}

/* lerp(v0, v1, t) = fma(t, v0, fma(-t, v1, v1)): include/cuda/cuda_utils.hpp:43-46 */
static inline real lerp_(real v0, real v1, real t) { return FMA_(t, v0, FMA_(-t, v1, v1)); }

/* Square root rounded toward -inf.  For the float build: the double sqrt of a
 * float is never exactly a float unless the float result is exact, so rounding
 * the double result down gives the correctly rounded-down float. */
static inline real sqrt_rd_(real s) {
#if defined(FRO_DOUBLE)
    return sqrt(s);
#else
    if (!(s > 0.f) || isinf(s)) return sqrtf(s);
    double d = sqrt((double)s);
    float r = (float)d;
    if ((double)r > d) r = nextafterf(r, 0.f);
    return r;
#endif
}

/* ------------------------------------------------------------------------- */
/* Trilinear sampling, include/cuda/cuda_utils.hpp:60-136                     */
/* ------------------------------------------------------------------------- */

typedef struct {
    int gx, gy, gz;
    real a, b, c;
} fro_cell;

/* clamp to [0, dim-1] (fminf(fmaxf(0, p), dim-1)), floor, fractional parts */
static inline void locate_(const fro_dims *d, real px, real py, real pz, fro_cell *cl) {
    real cx = FMIN_(FMAX_(R(0), px), (real)(d->X - 1));
    real cy = FMIN_(FMAX_(R(0), py), (real)(d->Y - 1));
    real cz = FMIN_(FMAX_(R(0), pz), (real)(d->Z - 1));
    cl->gx = (int)FLOOR_(cx);
    cl->gy = (int)FLOOR_(cy);
    cl->gz = (int)FLOOR_(cz);
    cl->a = cx - (real)cl->gx;
    cl->b = cy - (real)cl->gy;
    cl->c = cz - (real)cl->gz;
}

/* Corner reads of the Volume/VectorField operator() (include/cuda/device.hpp:17-19,
 * src/fastreg/cuda/vector_fields.cu:20-22): the linear index is formed without a
 * bounds check, so the +1 corner of a cell on the upper face aliases into the next
 * row/slice.  Those corners always carry weight 0.  The aliased linear index is
 * kept; an index past the end of the array (undefined in the reference) is clamped
 * to the last voxel. */
static inline real tri_unchecked_(const real *F, const fro_dims *d, const fro_cell *cl) {
    const int64_t N = nvox(d), X = d->X, XY = (int64_t)d->X * d->Y;
    const int64_t b = lin(d, cl->gx, cl->gy, cl->gz);
#define UC(dx, dy, dz) F[(b + (dx) + X * (dy) + XY * (dz)) < N ? (b + (dx) + X * (dy) + XY * (dz)) : N - 1]
    real r = lerp_(lerp_(lerp_(UC(1, 1, 1), UC(1, 1, 0), cl->c), lerp_(UC(1, 0, 1), UC(1, 0, 0), cl->c), cl->b),
                   lerp_(lerp_(UC(0, 1, 1), UC(0, 1, 0), cl->c), lerp_(UC(0, 0, 1), UC(0, 0, 0), cl->c), cl->b),
                   cl->a);
#undef UC
    return r;
}

/* Corner reads through get_global_idx (include/cuda/cuda_utils.hpp:31-37,109-136):
 * a corner outside the grid reads element 0 of the field. */
static inline real tri_checked_(const real *F, const fro_dims *d, const fro_cell *cl) {
    const int64_t X = d->X, XY = (int64_t)d->X * d->Y;
    const int64_t b = lin(d, cl->gx, cl->gy, cl->gz);
    const int ox = cl->gx + 1 < d->X, oy = cl->gy + 1 < d->Y, oz = cl->gz + 1 < d->Z;
#define CC(dx, dy, dz) \
    ((((dx) == 0 || ox) && ((dy) == 0 || oy) && ((dz) == 0 || oz)) ? F[b + (dx) + X * (dy) + XY * (dz)] : F[0])
    real r = lerp_(lerp_(lerp_(CC(1, 1, 1), CC(1, 1, 0), cl->c), lerp_(CC(1, 0, 1), CC(1, 0, 0), cl->c), cl->b),
                   lerp_(lerp_(CC(0, 1, 1), CC(0, 1, 0), cl->c), lerp_(CC(0, 0, 1), CC(0, 0, 0), cl->c), cl->b),
                   cl->a);
#undef CC
    return r;
}

/* apply_kernel (src/fastreg/cuda/vector_fields.cu:81-99) with interpolate_intensity
 * (include/cuda/cuda_utils.hpp:60-84): trilinear intensity at pos, label of the
 * floor corner of the clamped position.  pos is a 3-plane position field. */
void FN(warp)(const int *dims, const real *pos, const real *img, const int16_t *lab, real *out_img,
              int16_t *out_lab) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        fro_cell cl;
        locate_(&d, pos[i], pos[N + i], pos[2 * N + i], &cl);
        out_img[i] = tri_unchecked_(img, &d, &cl);
        if (out_lab) out_lab[i] = lab[lin(&d, cl.gx, cl.gy, cl.gz)];
    }
}

/* estimate_inverse (src/fastreg/cuda/vector_fields.cu:109-136; the reference's
 * registration never calls it): `sweeps` passes (48 in the reference) of
 *   psi_inv(x) <- -interpolate_field(psi, trunc(psi_inv(x)))
 * over every voxel, in place.  interpolate_field is the unchecked vector trilinear
 * sample (include/cuda/cuda_utils.hpp:86-107) and trunc keeps x, y, z
 * (cuda_utils.hpp:264).  A voxel's update reads only its own previous value (the
 * gather is from psi), so its sweeps can run back to back. */
void FN(estimate_inverse)(const int *dims, const real *psi, real *psi_inv, int sweeps) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        real p[3] = {psi_inv[i], psi_inv[N + i], psi_inv[2 * N + i]};
        for (int s = 0; s < sweeps; ++s) {
            fro_cell cl;
            locate_(&d, p[0], p[1], p[2], &cl);
            real q[3];
            for (int c = 0; c < 3; ++c) q[c] = R(-1) * tri_unchecked_(psi + c * N, &d, &cl);
            for (int c = 0; c < 3; ++c) p[c] = q[c];
        }
        for (int c = 0; c < 3; ++c) psi_inv[c * N + i] = p[c];
    }
}

/* interpolate_gradient (src/fastreg/cuda/vector_fields.cu:194-225; not called by the
 * reference's registration): out(x) = interpolate_field(field, trunc(pos(x))) over
 * every voxel, for any 3-component field. */
void FN(interpolate_field)(const int *dims, const real *field, const real *pos, real *out) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) {
        fro_cell cl;
        locate_(&d, pos[i], pos[N + i], pos[2 * N + i], &cl);
        for (int c = 0; c < 3; ++c) out[c * N + i] = tri_unchecked_(field + c * N, &d, &cl);
    }
}

/* ------------------------------------------------------------------------- */
/* Reference mode: one iteration of estimate_psi (solver.cu:329-433)          */
/* ------------------------------------------------------------------------- */

typedef struct {
    real alpha; /* ALPHA */
    real f1;    /* (p + 1) / t              solver.cu:198,205 */
    real m2;    /* C * p^2 * t^(p - 2)      solver.cu:199 */
    real tau;   /* TAU */
    real w_reg; /* W_REG */
} fro_ref_coef;

/* L = -(sum of 6 neighbours - 6 psi) on the interior, 0 elsewhere:
 * SecondOrderDifferentiator::laplacian, vector_fields.cu:275-300 */
void FN(ref_laplacian)(const int *dims, const real *psi, real *L) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d), X = d.X, XY = (int64_t)d.X * d.Y;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                for (int c = 0; c < 3; ++c) {
                    const real *P = psi + c * N;
                    if (!is_interior(&d, x, y, z)) {
                        L[c * N + i] = R(0);
                        continue;
                    }
                    real s = R(-6) * P[i];
                    s = s + P[i + 1];
                    s = s + P[i - 1];
                    s = s + P[i + X];
                    s = s + P[i - X];
                    s = s + P[i + XY];
                    s = s + P[i - XY];
                    L[c * N + i] = R(-1) * s;
                }
            }
}

/* det(Mat4f) exactly as written in include/cuda/cuda_utils.hpp:389-396
 * (mis-parenthesised: the second triple product is (m02*m11 + m20)*(m12*m21*m00)). */
static inline real det_ref_(const real m[3][3]) {
    real first = ((m[0][0] * m[1][1]) * m[2][2] + (m[1][0] * m[2][1]) * m[0][2]) + (m[2][0] * m[0][1]) * m[1][2];
    real second = ((m[0][2] * m[1][1]) + m[2][0]) * ((m[1][2] * m[2][1]) * m[0][0]) + (m[2][2] * m[0][1]) * m[1][0];
    return first - second;
}

/* One voxel of the fused pass A: divergence + density (solver.cu:101-173),
 * Jacobian of psi_inv (vector_fields.cu:503-535), potential gradient
 * (solver.cu:56-80), (Dv)v (vector_fields.cu:352-404), upwind velocity
 * Laplacian (vector_fields.cu:307-346), velocity update (solver.cu:188-211),
 * psi_inv update (solver.cu:263-279). */
static void ref_pass_a_voxel_(const fro_dims *d, const fro_ref_coef *k, const real *S, const real *T,
                              int first_iter, const real *rho, const real *v, const real *pinv, const real *L,
                              real *rho_n, real *v_n, real *pinv_n, int x, int y, int z) {
    const int64_t N = nvox(d), X = d->X, XY = (int64_t)d->X * d->Y;
    const int64_t i = lin(d, x, y, z);
    const real *vx_ = v, *vy_ = v + N, *vz_ = v + 2 * N;

    /* --- divergence of rho*v (upwind) and density update --- */
    const real vx = vx_[i], vy = vy_[i], vz = vz_[i];
    const real p = rho[i];
    real t11 = (vx > R(0)) ? (-vx) * p : (-vx) * rho[i + 1];
    real vxm = vx_[i - 1];
    real t12 = (vxm > R(0)) ? vxm * rho[i - 1] : vxm * p;
    real t21 = (vy > R(0)) ? (-vy) * p : (-vy) * rho[i + X];
    real vym = vy_[i - X];
    real t22 = (vym > R(0)) ? vym * rho[i - X] : vym * p;
    real t31 = (vz > R(0)) ? (-vz) * p : (-vz) * rho[i + XY];
    real vzm = vz_[i - XY];
    real t32 = (vzm > R(0)) ? vzm * rho[i - XY] : vzm * p;
    real div = ((((t11 + t12) + t21) + t22) + t31) + t32;
    real rho_new = p + k->alpha * div;
    rho_n[i] = rho_new;

    /* --- Jacobian of psi_inv: row r = d(psi_inv_r)/d(x,y,z) --- */
    real M[3][3];
    for (int r = 0; r < 3; ++r) {
        const real *P = pinv + r * N;
        M[r][0] = (P[i + 1] - P[i - 1]) * R(0.5);
        M[r][1] = (P[i + X] - P[i - X]) * R(0.5);
        M[r][2] = (P[i + XY] - P[i - XY]) * R(0.5);
    }
    const real det = det_ref_(M);

    /* --- T o psi_inv and L o psi_inv at psi_inv(x) --- */
    fro_cell cl;
    locate_(d, pinv[i], pinv[N + i], pinv[2 * N + i], &cl);
    const real Tq = first_iter ? T[i] : tri_unchecked_(T, d, &cl);
    real Lq[3];
    for (int c = 0; c < 3; ++c) Lq[c] = tri_unchecked_(L + c * N, d, &cl);

    /* --- gradient of S (central differences), potential gradient --- */
    real gs[3];
    gs[0] = (S[i + 1] - S[i - 1]) * R(0.5);
    gs[1] = (S[i + X] - S[i - X]) * R(0.5);
    gs[2] = (S[i + XY] - S[i - XY]) * R(0.5);
    const real diff = S[i] - Tq;
    real gU[3];
    for (int c = 0; c < 3; ++c) gU[c] = ((diff * gs[c]) + (k->w_reg * Lq[c])) * det;

    /* --- (Dv)v: entropy scheme on the diagonal, upwind off the diagonal --- */
    const real vxp_x = vx_[i + 1], vyp_y = vy_[i + X], vzp_z = vz_[i + XY];
    real ax1 = ((FMAX_(vx, R(0)) * FMAX_(vx, R(0)) - FMIN_(vx, R(0)) * FMIN_(vx, R(0))) +
                FMIN_(vxp_x, R(0)) * FMIN_(vxp_x, R(0))) -
               FMAX_(vxp_x, R(0)) * FMAX_(vxp_x, R(0));
    real ax2 = (vy > R(0)) ? vy * (vx - vx_[i - X]) : vy * (vx_[i + X] - vx);
    real ax3 = (vz > R(0)) ? vz * (vx - vx_[i - XY]) : vz * (vx_[i + XY] - vx);
    real ay1 = (vx > R(0)) ? vx * (vy - vy_[i - 1]) : vx * (vy_[i + 1] - vy);
    real ay2 = ((FMAX_(vy, R(0)) * FMAX_(vy, R(0)) - FMIN_(vy, R(0)) * FMIN_(vy, R(0))) +
                FMIN_(vyp_y, R(0)) * FMIN_(vyp_y, R(0))) -
               FMAX_(vyp_y, R(0)) * FMAX_(vyp_y, R(0));
    real ay3 = (vz > R(0)) ? vz * (vy - vy_[i - XY]) : vz * (vy_[i + XY] - vy);
    real az1 = (vx > R(0)) ? vx * (vz - vz_[i - 1]) : vx * (vz_[i + 1] - vz);
    real az2 = (vy > R(0)) ? vy * (vz - vz_[i - X]) : vy * (vz_[i + X] - vz);
    real az3 = ((FMAX_(vz, R(0)) * FMAX_(vz, R(0)) - FMIN_(vz, R(0)) * FMIN_(vz, R(0))) +
                FMIN_(vzp_z, R(0)) * FMIN_(vzp_z, R(0))) -
               FMAX_(vzp_z, R(0)) * FMAX_(vzp_z, R(0));
    real dvv[3];
    dvv[0] = (R(0.5) * ax1 + ax2) + ax3;
    dvv[1] = (ay1 + R(0.5) * ay2) + ay3;
    dvv[2] = (az1 + az2) + R(0.5) * az3;

    /* --- delta_v: negated upwind second differences on x in [2,X-3],
     *     y in [2,Y-2], z in [2,Z-3]; the y and z "forward" branches read
     *     (+2, -1, 0) as written (vector_fields.cu:320-332).  At y = Y-2 the
     *     unchecked y+2 read lands on linear index i + 2X = voxel (x, 0, z+1),
     *     which is inside the array; that aliased value is used as is. --- */
    real dv[3] = {R(0), R(0), R(0)};
    if (x >= 2 && x <= d->X - 3 && y >= 2 && y <= d->Y - 2 && z >= 2 && z <= d->Z - 3) {
        const real vel[3] = {vx, vy, vz};
        for (int c = 0; c < 3; ++c) {
            const real *V = v + c * N;
            real xx = (vx < R(0)) ? (V[i + 2] - R(2) * V[i + 1]) + vel[c] : (vel[c] - R(2) * V[i - 1]) + V[i - 2];
            real yy = (vy < R(0)) ? (V[i + 2 * X] - R(2) * V[i - X]) + vel[c]
                                  : (vel[c] - R(2) * V[i - X]) + V[i - 2 * X];
            real zz = (vz < R(0)) ? (V[i + 2 * XY] - R(2) * V[i - XY]) + vel[c]
                                  : (vel[c] - R(2) * V[i - XY]) + V[i - 2 * XY];
            dv[c] = R(-1) * ((xx + yy) + zz);
        }
    }

    /* --- velocity update --- */
    const real q = k->m2 / (FABS_(rho_new) + R(1e-5));
    const real vel[3] = {vx, vy, vz};
    real vn[3];
    for (int c = 0; c < 3; ++c) {
        real friction = k->f1 * vel[c];
        real diffusion = k->tau * dv[c];
        real potential = q * gU[c];
        real acc = ((friction + dvv[c]) - diffusion) + potential;
        vn[c] = vel[c] - k->alpha * acc;
        v_n[c * N + i] = vn[c];
    }

    /* --- psi_inv update with J(psi_inv) * v_new at x --- */
    for (int r = 0; r < 3; ++r) {
        real jv = ((M[r][0] * vn[0]) + (M[r][1] * vn[1])) + (M[r][2] * vn[2]);
        pinv_n[r * N + i] = pinv[r * N + i] - k->alpha * jv;
    }
}

/* Pass A over the interior.  rho_n/v_n/pinv_n must already hold the boundary
 * values (the boundary never changes). */
void FN(ref_pass_a)(const int *dims, const fro_ref_coef *k, const real *S, const real *T, int first_iter,
                    const real *rho, const real *v, const real *pinv, const real *L, real *rho_n, real *v_n,
                    real *pinv_n) {
    fro_dims d = {dims[0], dims[1], dims[2]};
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.Z - 1; ++z)
        for (int y = 1; y < d.Y - 1; ++y)
            for (int x = 1; x < d.X - 1; ++x)
                ref_pass_a_voxel_(&d, k, S, T, first_iter, rho, v, pinv, L, rho_n, v_n, pinv_n, x, y, z);
}

/* Pass B: psi += alpha * v o psi on the interior (solver.cu:230-247); returns the
 * max update norm and its linear index (ties -> lowest index; boundary updates
 * count as 0). */
void FN(ref_pass_b)(const int *dims, real alpha, const real *v, real *psi, real *max_norm, int64_t *argmax) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    real best = R(0);
    int64_t best_i = 0;
#pragma omp parallel
    {
        real lbest = R(0);
        int64_t lbest_i = INT64_MAX;
#pragma omp for schedule(static)
        for (int z = 1; z < d.Z - 1; ++z)
            for (int y = 1; y < d.Y - 1; ++y)
                for (int x = 1; x < d.X - 1; ++x) {
                    int64_t i = lin(&d, x, y, z);
                    fro_cell cl;
                    locate_(&d, psi[i], psi[N + i], psi[2 * N + i], &cl);
                    real up[3];
                    for (int c = 0; c < 3; ++c) {
                        up[c] = alpha * tri_checked_(v + c * N, &d, &cl);
                        psi[c * N + i] = psi[c * N + i] + up[c];
                    }
                    real nrm = sqrt_rd_((up[0] * up[0] + up[1] * up[1]) + up[2] * up[2]);
                    if (nrm > lbest || (nrm == lbest && i < lbest_i)) {
                        lbest = nrm;
                        lbest_i = i;
                    }
                }
#pragma omp critical
        {
            if (lbest > best || (lbest == best && lbest_i < best_i && lbest > R(0))) {
                best = lbest;
                best_i = lbest_i;
            }
        }
    }
    *max_norm = best;
    *argmax = best_i;
}

/* Scalars of one iteration: solver.cu:198-199 with t as scheduled in 428-432. */
void FN(ref_coef)(real alpha, real t, real p, real C, real tau, real w_reg, fro_ref_coef *k) {
    real m1 = p + R(1);
#if defined(FRO_DOUBLE)
    real m2 = (C * pow(p, 2.0)) * pow(t, p - 2.0);
#else
    real m2 = (C * powf(p, 2.f)) * powf(t, p - 2.f);
#endif
    k->alpha = alpha;
    k->f1 = m1 / t;
    k->m2 = m2;
    k->tau = tau;
    k->w_reg = w_reg;
}

typedef struct {
    int max_iter;
    int reset_iter;
    real max_update_norm;
    real rho_0, tau, w_reg, alpha, p, C;
    int keep_state; /* 1: continue from the given psi/psi_inv/v (reference carry-over) */
} fro_ref_params;

/* Full reference-mode registration (estimate_psi, solver.cu:295-444; the
 * identity/zero/rho_0 start of fastreg.cpp:24-46, solver.cpp:56-63).
 * State arrays (rho N, v/psi/psi_inv 3N) are in/out.  Returns the number of
 * iterations run; max-norm trace (max_iter entries) and final outputs. */
int FN(ref_register)(const int *dims, const fro_ref_params *P, const real *T, const int16_t *labT, const real *S,
                     const int16_t *labS, real *rho, real *v, real *psi, real *psi_inv, real *out_T,
                     int16_t *out_labT, real *out_S, int16_t *out_labS, real *trace_norm, int64_t *trace_idx,
                     int *converged) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    if (!P->keep_state) {
        for (int64_t i = 0; i < N; ++i) rho[i] = P->rho_0;
        memset(v, 0, sizeof(real) * 3 * N);
        for (int z = 0; z < d.Z; ++z)
            for (int y = 0; y < d.Y; ++y)
                for (int x = 0; x < d.X; ++x) {
                    int64_t i = lin(&d, x, y, z);
                    psi[i] = psi_inv[i] = (real)x;
                    psi[N + i] = psi_inv[N + i] = (real)y;
                    psi[2 * N + i] = psi_inv[2 * N + i] = (real)z;
                }
    } else {
        for (int64_t i = 0; i < N; ++i) rho[i] = P->rho_0; /* init_density_kernel, solver.cu:317 */
    }
    real *L = (real *)malloc(sizeof(real) * 3 * N);
    real *rho2 = (real *)malloc(sizeof(real) * N);
    real *v2 = (real *)malloc(sizeof(real) * 3 * N);
    real *pinv2 = (real *)malloc(sizeof(real) * 3 * N);
    memcpy(rho2, rho, sizeof(real) * N);
    memcpy(v2, v, sizeof(real) * 3 * N);
    memcpy(pinv2, psi_inv, sizeof(real) * 3 * N);
    real *r0 = rho, *r1 = rho2, *v0 = v, *v1 = v2, *q0 = psi_inv, *q1 = pinv2;

    real t = P->alpha;
    int iter = 1, ran = 0;
    *converged = 0;
    while (iter <= P->max_iter) {
        fro_ref_coef k;
        FN(ref_coef)(P->alpha, t, P->p, P->C, P->tau, P->w_reg, &k);
        FN(ref_laplacian)(dims, psi, L);
        FN(ref_pass_a)(dims, &k, S, T, iter == 1, r0, v0, q0, L, r1, v1, q1);
        real *tmp;
        tmp = r0; r0 = r1; r1 = tmp;
        tmp = v0; v0 = v1; v1 = tmp;
        tmp = q0; q0 = q1; q1 = tmp;
        real mx;
        int64_t am;
        FN(ref_pass_b)(dims, P->alpha, v0, psi, &mx, &am);
        if (trace_norm) trace_norm[iter - 1] = mx;
        if (trace_idx) trace_idx[iter - 1] = am;
        ran = iter;
        if (mx <= P->max_update_norm) {
            *converged = 1;
            break;
        }
        if (iter == P->max_iter) break;
        iter++;
        t += P->alpha;
        if (P->reset_iter > 0 && iter % P->reset_iter == 0) t = P->alpha;
    }
    /* results live in r0/v0/q0; copy back into the caller's arrays */
    if (r0 != rho) memcpy(rho, r0, sizeof(real) * N);
    if (v0 != v) memcpy(v, v0, sizeof(real) * 3 * N);
    if (q0 != psi_inv) memcpy(psi_inv, q0, sizeof(real) * 3 * N);
    free(L);
    free(rho2);
    free(v2);
    free(pinv2);

    /* final warps: T o psi_inv (solver.cu:402, or T itself if no iteration ran)
     * and S o psi (solver.cu:435) */
    if (ran == 0) {
        memcpy(out_T, T, sizeof(real) * N);
        memcpy(out_labT, labT, sizeof(int16_t) * N);
    } else {
        FN(warp)(dims, psi_inv, T, labT, out_T, out_labT);
    }
    FN(warp)(dims, psi, S, labS, out_S, out_labS);
    return ran;
}

/* ------------------------------------------------------------------------- */
/* Statistics: energy, deformation Jacobian, fold count, Dice                 */
/* ------------------------------------------------------------------------- */

/* Jacobian of the displacement u = psi - x with the mirrored one-sided boundary
 * of Differentiator::deformation_jacobian (vector_fields.cu:537-585); row r =
 * d(u_r)/d(x,y,z). */
static inline void deformation_jacobian_(const fro_dims *d, const real *psi, int x, int y, int z, real J[3][3]) {
    const int64_t N = nvox(d);
    int x1 = x + 1, x2 = x - 1, y1 = y + 1, y2 = y - 1, z1 = z + 1, z2 = z - 1;
    if (x == 0) x2 = x + 1; else if (x == d->X - 1) x1 = x - 1;
    if (y == 0) y2 = y + 1; else if (y == d->Y - 1) y1 = y - 1;
    if (z == 0) z2 = z + 1; else if (z == d->Z - 1) z1 = z - 1;
    const int64_t ix1 = lin(d, x1, y, z), ix2 = lin(d, x2, y, z);
    const int64_t iy1 = lin(d, x, y1, z), iy2 = lin(d, x, y2, z);
    const int64_t iz1 = lin(d, x, y, z1), iz2 = lin(d, x, y, z2);
    const real cx1[3] = {(real)x1, (real)y, (real)z}, cx2[3] = {(real)x2, (real)y, (real)z};
    const real cy1[3] = {(real)x, (real)y1, (real)z}, cy2[3] = {(real)x, (real)y2, (real)z};
    const real cz1[3] = {(real)x, (real)y, (real)z1}, cz2[3] = {(real)x, (real)y, (real)z2};
    for (int r = 0; r < 3; ++r) {
        const real *P = psi + r * N;
        J[r][0] = ((P[ix1] - cx1[r]) - (P[ix2] - cx2[r])) * R(0.5);
        J[r][1] = ((P[iy1] - cy1[r]) - (P[iy2] - cy2[r])) * R(0.5);
        J[r][2] = ((P[iz1] - cz1[r]) - (P[iz2] - cz2[r])) * R(0.5);
    }
}

/* correct 3x3 determinant of F = I + J, fixed evaluation order */
static inline real det_true_(const real J[3][3]) {
    const real f00 = J[0][0] + R(1), f11 = J[1][1] + R(1), f22 = J[2][2] + R(1);
    const real f01 = J[0][1], f02 = J[0][2], f10 = J[1][0], f12 = J[1][2], f20 = J[2][0], f21 = J[2][1];
    const real c0 = f11 * f22 - f12 * f21;
    const real c1 = f10 * f22 - f12 * f20;
    const real c2 = f10 * f21 - f11 * f20;
    return (f00 * c0 - f01 * c1) + f02 * c2;
}

typedef struct {
    double e_data;  /* 0.5 * sum (T - S o psi)^2          reductor.cu:11-112, reductor.cpp:45-61 */
    double e_reg;   /* 0.5 * sum ||J_u||_F^2               reductor.cu:224-324 */
    int64_t folds;  /* #{det(I + J_u) <= 0} */
    int64_t dice_inter[256]; /* per label, over [0,X-1)x[0,Y-1)x[0,Z-1) (solver.cu:21-35) */
    int64_t dice_count[256];
    int64_t dice_out_of_range;
} fro_stats;

/* warped_S = S o psi, labels of both; psi positions. */
void FN(stats)(const int *dims, int no_labels, const real *T, const int16_t *labT, const real *warped_S,
               const int16_t *warped_labS, const real *psi, fro_stats *st) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    memset(st, 0, sizeof(*st));
    double ed = 0.0, er = 0.0;
    int64_t folds = 0;
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                real df = T[i] - warped_S[i];
                ed += (double)df * (double)df;
                real J[3][3];
                deformation_jacobian_(&d, psi, x, y, z, J);
                real r0 = (J[0][0] * J[0][0] + J[0][1] * J[0][1]) + J[0][2] * J[0][2];
                real r1 = (J[1][0] * J[1][0] + J[1][1] * J[1][1]) + J[1][2] * J[1][2];
                real r2 = (J[2][0] * J[2][0] + J[2][1] * J[2][1]) + J[2][2] * J[2][2];
                er += (double)((r0 + r1) + r2);
                if (det_true_(J) <= R(0)) folds++;
                if (x < d.X - 1 && y < d.Y - 1 && z < d.Z - 1) {
                    int la = warped_labS[i], lb = labT[i];
                    int oka = la >= 0 && la < no_labels && la < 256;
                    int okb = lb >= 0 && lb < no_labels && lb < 256;
                    if (!oka || !okb) {
                        st->dice_out_of_range++;
                        continue;
                    }
                    st->dice_count[la]++;
                    st->dice_count[lb]++;
                    if (la == lb) st->dice_inter[la]++;
                }
            }
    st->e_data = 0.5 * ed;
    st->e_reg = 0.5 * er;
    st->folds = folds;
}

/* Per-voxel fields used by the parity tests: deformation Jacobian (9 planes,
 * row-major r*3+c) and det(I + J_u). */
void FN(deformation_jacobian)(const int *dims, const real *psi, real *J9, real *detF) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                real J[3][3];
                deformation_jacobian_(&d, psi, x, y, z, J);
                if (J9)
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) J9[(r * 3 + c) * N + i] = J[r][c];
                if (detF) detF[i] = det_true_(J);
            }
}

/* the reference's det as a per-voxel field of J(psi_inv) (interior; 0 outside),
 * for the known-answer tests of the mis-parenthesised determinant */
void FN(ref_det_field)(const int *dims, const real *pinv, real *out) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d), X = d.X, XY = (int64_t)d.X * d.Y;
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                if (!is_interior(&d, x, y, z)) {
                    out[i] = R(0);
                    continue;
                }
                real M[3][3];
                for (int r = 0; r < 3; ++r) {
                    const real *P = pinv + r * N;
                    M[r][0] = (P[i + 1] - P[i - 1]) * R(0.5);
                    M[r][1] = (P[i + X] - P[i - X]) * R(0.5);
                    M[r][2] = (P[i + XY] - P[i - XY]) * R(0.5);
                }
                out[i] = det_ref_(M);
            }
}

/* ------------------------------------------------------------------------- */
/* Sobolev solver (no counterpart in the reference; see fr_sob.h)             */
/* ------------------------------------------------------------------------- */

/* Gaussian taps exp(-k^2/(2 sigma^2)), normalised, computed in double. */
void FN(gaussian_taps)(double sigma, int width, real *taps) {
    int R = width / 2;
    double w[64], sum = 0.0;
    for (int k = -R; k <= R; ++k) {
        w[k + R] = exp(-(double)k * (double)k / (2.0 * sigma * sigma));
        sum += w[k + R];
    }
    for (int k = 0; k < width; ++k) taps[k] = (real)(w[k] / sum);
}

typedef struct {
    int64_t base;
    real a, b, c;
    int in_x, in_y, in_z;
} fro_scell;

static inline void sob_locate_(const fro_dims *d, real px, real py, real pz, fro_scell *s) {
    real cx = FMIN_(FMAX_(R(0), px), (real)(d->X - 1));
    real cy = FMIN_(FMAX_(R(0), py), (real)(d->Y - 1));
    real cz = FMIN_(FMAX_(R(0), pz), (real)(d->Z - 1));
    int gx = (int)FLOOR_(cx), gy = (int)FLOOR_(cy), gz = (int)FLOOR_(cz);
    if (gx > d->X - 2) gx = d->X - 2;
    if (gy > d->Y - 2) gy = d->Y - 2;
    if (gz > d->Z - 2) gz = d->Z - 2;
    s->a = cx - (real)gx;
    s->b = cy - (real)gy;
    s->c = cz - (real)gz;
    s->in_x = px >= R(0) && px <= (real)(d->X - 1);
    s->in_y = py >= R(0) && py <= (real)(d->Y - 1);
    s->in_z = pz >= R(0) && pz <= (real)(d->Z - 1);
    s->base = lin(d, gx, gy, gz);
}

/* Graph Laplacian of the displacement u = phi - x over the grid's neighbours (the
 * gradient of 0.5 * sum over grid edges |u(x) - u(q)|^2): for each neighbour q inside the
 * grid, in the order -x, +x, -y, +y, -z, +z, lap_c += (phi_c(x) - phi_c(q)) + (q - x)_c. */
static inline void lap_u_(const fro_dims *d, const real *phi, int x, int y, int z, real out[3]) {
    const int64_t N = nvox(d), i = lin(d, x, y, z);
    const int64_t X = d->X, XY = (int64_t)d->X * d->Y;
    const int ok[6] = {x > 0, x < d->X - 1, y > 0, y < d->Y - 1, z > 0, z < d->Z - 1};
    const int64_t off[6] = {-1, 1, -X, X, -XY, XY};
    for (int c = 0; c < 3; ++c) {
        real acc = R(0);
        for (int k = 0; k < 6; ++k) {
            if (!ok[k]) continue;
            const real delta = (k / 2 == c) ? ((k & 1) ? R(1) : R(-1)) : R(0);
            acc = acc + ((phi[c * N + i] - phi[c * N + i + off[k]]) + delta);
        }
        out[c] = acc;
    }
}

/* g = (W - T) * dW/dphi + lambda * lap(u) with W = S(phi) trilinear; returns 0.5 * sum (W - T)^2 */
double FN(sob_grad)(const int *dims, const real *S, const real *T, const real *phi, real lambda, real *g,
                    real *W_out) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d), X = d.X, XY = (int64_t)d.X * d.Y;
    /* per-slice partial sums added in slice order: the same energy for any thread count */
    double *part = (double *)calloc((size_t)d.Z, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int zz = 0; zz < d.Z; ++zz) {
        double ez = 0.0;
        for (int64_t i = zz * XY; i < (zz + 1) * XY; ++i) {
            fro_scell s;
            sob_locate_(&d, phi[i], phi[N + i], phi[2 * N + i], &s);
            const int64_t b = s.base;
            const real f000 = S[b], f100 = S[b + 1], f010 = S[b + X], f110 = S[b + 1 + X];
            const real f001 = S[b + XY], f101 = S[b + 1 + XY], f011 = S[b + X + XY], f111 = S[b + 1 + X + XY];
            const real e11 = lerp_(f111, f110, s.c), e10 = lerp_(f101, f100, s.c);
            const real e01 = lerp_(f011, f010, s.c), e00 = lerp_(f001, f000, s.c);
            const real A1 = lerp_(e11, e10, s.b), A0 = lerp_(e01, e00, s.b);
            const real W = lerp_(A1, A0, s.a);
            const real dWa = s.in_x ? A1 - A0 : R(0);
            const real dWb = s.in_y ? lerp_(e11 - e10, e01 - e00, s.a) : R(0);
            const real dWc = s.in_z ? lerp_(lerp_(f111 - f110, f101 - f100, s.b), lerp_(f011 - f010, f001 - f000, s.b), s.a)
                                    : R(0);
            const real r = W - T[i];
            const int z = (int)(i / XY), y = (int)((i - z * XY) / X), x = (int)(i - z * XY - y * X);
            real lap[3];
            lap_u_(&d, phi, x, y, z, lap);
            g[i] = (r * dWa) + (lambda * lap[0]);
            g[N + i] = (r * dWb) + (lambda * lap[1]);
            g[2 * N + i] = (r * dWc) + (lambda * lap[2]);
            if (W_out) W_out[i] = W;
            ez += (double)r * (double)r;
        }
        part[zz] = ez;
    }
    double e = 0.0;
    for (int zz = 0; zz < d.Z; ++zz) e += part[zz];
    free(part);
    return 0.5 * e;
}

/* one separable pass along axis with the replicate boundary, each tap a fused
 * multiply-add in the order -R..R; momentum != 0: m = damping * m - step * (smoothed src) */
void FN(sob_smooth)(const int *dims, const real *taps, int R_, int axis, const real *src, real *dst, int momentum,
                    real damping, real step) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    const int dim = axis == 0 ? d.X : (axis == 1 ? d.Y : d.Z);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)d.X : (int64_t)d.X * d.Y);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                const int64_t i = lin(&d, x, y, z);
                const int pos = axis == 0 ? x : (axis == 1 ? y : z);
                for (int c = 0; c < 3; ++c) {
                    const real *Sp = src + c * N;
                    real acc = R(0);
                    for (int k = -R_; k <= R_; ++k) {
                        int q = pos + k;
                        if (q < 0) q = 0;
                        if (q > dim - 1) q = dim - 1;
                        acc = FMA_(taps[k + R_], Sp[i + (int64_t)(q - pos) * stride], acc);
                    }
                    if (momentum)
                        dst[c * N + i] = damping * dst[c * N + i] - step * acc;
                    else
                        dst[c * N + i] = acc;
                }
            }
}

/* phi += m(phi) (trilinear, sobolev cell); returns max |update| and its index */
void FN(sob_pass_b)(const int *dims, const real *m, real *phi, real *max_norm, int64_t *argmax) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d), X = d.X, XY = (int64_t)d.X * d.Y;
    real best = R(0);
    int64_t best_i = 0;
    /* per-thread first maximum (the gather reads m, never phi), merged so that ties go to
     * the lowest index: the result of the serial loop with its strict '>' */
#pragma omp parallel
    {
        real lbest = R(0);
        int64_t lbest_i = INT64_MAX;
#pragma omp for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            fro_scell s;
            sob_locate_(&d, phi[i], phi[N + i], phi[2 * N + i], &s);
            const int64_t b = s.base;
            real u[3];
            for (int c = 0; c < 3; ++c) {
                const real *F = m + c * N;
                u[c] = lerp_(lerp_(lerp_(F[b + 1 + X + XY], F[b + 1 + X], s.c), lerp_(F[b + 1 + XY], F[b + 1], s.c), s.b),
                             lerp_(lerp_(F[b + X + XY], F[b + X], s.c), lerp_(F[b + XY], F[b], s.c), s.b), s.a);
            }
            for (int c = 0; c < 3; ++c) phi[c * N + i] = phi[c * N + i] + u[c];
            real nrm = sqrt_rd_((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
            if (nrm > lbest) {
                lbest = nrm;
                lbest_i = i;
            }
        }
#pragma omp critical
        {
            if (lbest > best || (lbest == best && lbest_i < best_i && lbest > R(0))) {
                best = lbest;
                best_i = lbest_i;
            }
        }
    }
    *max_norm = best;
    *argmax = best_i;
}

typedef struct {
    int max_iter;
    real max_update_norm;
    real damping, step, sigma;
    int width;
    real lambda; /* W_REG: weight of the displacement's graph Laplacian */
} fro_sob_params;

/* full sobolev registration from phi = identity, m = 0; returns iterations run */
int FN(sob_register)(const int *dims, const fro_sob_params *P, const real *T, const real *S, real *phi, real *m,
                     real *trace_norm, int64_t *trace_idx, double *trace_energy, int *converged) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    real taps[64];
    FN(gaussian_taps)(P->sigma, P->width, taps);
    const int Rr = P->width / 2;
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                phi[i] = (real)x;
                phi[N + i] = (real)y;
                phi[2 * N + i] = (real)z;
            }
    memset(m, 0, sizeof(real) * 3 * N);
    real *g = (real *)malloc(sizeof(real) * 3 * N);
    real *tmp = (real *)malloc(sizeof(real) * 3 * N);
    int ran = 0;
    *converged = 0;
    for (int it = 1; it <= P->max_iter; ++it) {
        double e = FN(sob_grad)(dims, S, T, phi, P->lambda, g, NULL);
        if (trace_energy) trace_energy[it - 1] = e;
        FN(sob_smooth)(dims, taps, Rr, 0, g, tmp, 0, R(0), R(0));
        FN(sob_smooth)(dims, taps, Rr, 1, tmp, g, 0, R(0), R(0));
        FN(sob_smooth)(dims, taps, Rr, 2, g, m, 1, P->damping, P->step);
        real mx;
        int64_t am;
        FN(sob_pass_b)(dims, m, phi, &mx, &am);
        if (trace_norm) trace_norm[it - 1] = mx;
        if (trace_idx) trace_idx[it - 1] = am;
        ran = it;
        if (mx <= P->max_update_norm) {
            *converged = 1;
            break;
        }
    }
    free(g);
    free(tmp);
    return ran;
}

/* label of the voxel nearest to each position (clamped, round half up) */
void FN(warp_nearest_label)(const int *dims, const real *pos, const int16_t *lab, int16_t *out_lab) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    for (int64_t i = 0; i < N; ++i) {
        real cx = FMIN_(FMAX_(R(0), pos[i]), (real)(d.X - 1));
        real cy = FMIN_(FMAX_(R(0), pos[N + i]), (real)(d.Y - 1));
        real cz = FMIN_(FMAX_(R(0), pos[2 * N + i]), (real)(d.Z - 1));
        int ix = (int)FLOOR_(cx + R(0.5)), iy = (int)FLOOR_(cy + R(0.5)), iz = (int)FLOOR_(cz + R(0.5));
        if (ix > d.X - 1) ix = d.X - 1;
        if (iy > d.Y - 1) iy = d.Y - 1;
        if (iz > d.Z - 1) iz = d.Z - 1;
        out_lab[i] = lab[lin(&d, ix, iy, iz)];
    }
}

/* ------------------------------------------------------------------------- */
/* Differentiated sobolev registration (the adjoint of the loop above)        */
/* ------------------------------------------------------------------------- */

/* trilinear weights of the 8 corners (order 000,100,010,110,001,101,011,111 by
 * (dx,dy,dz)), value, position derivative (masked on clamped axes) and Hessian */
typedef struct {
    real w[8];
    int64_t off[8];
    real val, d[3], H[3][3];
} fro_tri;

static void tri_eval_(const fro_dims *d, const real *F, const fro_scell *s, fro_tri *t, int want_hessian) {
    const int64_t X = d->X, XY = (int64_t)d->X * d->Y, b = s->base;
    const int64_t off[8] = {0, 1, X, 1 + X, XY, 1 + XY, X + XY, 1 + X + XY};
    real f[8];
    for (int q = 0; q < 8; ++q) {
        t->off[q] = b + off[q];
        f[q] = F ? F[b + off[q]] : R(0);
    }
    const real a = s->a, bb = s->b, c = s->c;
    for (int q = 0; q < 8; ++q) {
        const real wx = (q & 1) ? a : R(1) - a, wy = (q & 2) ? bb : R(1) - bb, wz = (q & 4) ? c : R(1) - c;
        t->w[q] = wx * wy * wz;
    }
    if (!F) return;
    const real f000 = f[0], f100 = f[1], f010 = f[2], f110 = f[3], f001 = f[4], f101 = f[5], f011 = f[6], f111 = f[7];
    const real e11 = lerp_(f111, f110, c), e10 = lerp_(f101, f100, c);
    const real e01 = lerp_(f011, f010, c), e00 = lerp_(f001, f000, c);
    const real A1 = lerp_(e11, e10, bb), A0 = lerp_(e01, e00, bb);
    t->val = lerp_(A1, A0, a);
    const real d11 = f111 - f110, d10 = f101 - f100, d01 = f011 - f010, d00 = f001 - f000;
    t->d[0] = s->in_x ? A1 - A0 : R(0);
    t->d[1] = s->in_y ? lerp_(e11 - e10, e01 - e00, a) : R(0);
    t->d[2] = s->in_z ? lerp_(lerp_(d11, d10, bb), lerp_(d01, d00, bb), a) : R(0);
    if (!want_hessian) return;
    const int in[3] = {s->in_x, s->in_y, s->in_z};
    real H01 = (e11 - e10) - (e01 - e00);
    real H02 = lerp_(d11, d10, bb) - lerp_(d01, d00, bb);
    real H12 = lerp_(d11 - d10, d01 - d00, a);
    memset(t->H, 0, sizeof(t->H));
    if (in[0] && in[1]) t->H[0][1] = t->H[1][0] = H01;
    if (in[0] && in[2]) t->H[0][2] = t->H[2][0] = H02;
    if (in[1] && in[2]) t->H[1][2] = t->H[2][1] = H12;
}

/* out(x) = sum_k w_k in(clamp(x + k)) along axis: transpose, scatter form.  A
 * scatter stays on its line along `axis`, so lines are independent: the loop is split
 * over slices (axis x, y) or rows (axis z), and every line still receives its
 * contributions in increasing position -- the same sums for any thread count. */
static void smooth_t_(const fro_dims *d, const real *taps, int Rr, int axis, const real *src, real *dst) {
    const int64_t N = nvox(d);
    const int dim = axis == 0 ? d->X : (axis == 1 ? d->Y : d->Z);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)d->X : (int64_t)d->X * d->Y);
    memset(dst, 0, sizeof(real) * 3 * N);
    const int outer = axis == 2 ? d->Y : d->Z, inner = axis == 2 ? d->Z : d->Y;
#pragma omp parallel for schedule(static)
    for (int o = 0; o < outer; ++o)
        for (int n = 0; n < inner; ++n)
            for (int x = 0; x < d->X; ++x) {
                const int z = axis == 2 ? n : o, y = axis == 2 ? o : n;
                const int64_t i = lin(d, x, y, z);
                const int pos = axis == 0 ? x : (axis == 1 ? y : z);
                for (int k = -Rr; k <= Rr; ++k) {
                    int q = pos + k;
                    if (q < 0) q = 0;
                    if (q > dim - 1) q = dim - 1;
                    const int64_t j = i + (int64_t)(q - pos) * stride;
                    for (int c = 0; c < 3; ++c) dst[c * N + j] += taps[k + Rr] * src[c * N + i];
                }
            }
}

typedef struct {
    int iters;
    real damping, step, sigma;
    int width;
} fro_sobgrad_params;

/* J = 0.5 sum (S(phi_K) - T)^2 + 0.1 sum |m_K|^2 after K sobolev iterations from
 * phi_0 = identity, m_0 = v0, with regulariser weight lambda.  Returns J; with
 * grad_v0 != NULL also dJ/dv0 (3N) and dJ/dlambda (reverse mode, all states kept). */
double FN(sob_loss_grad)(const int *dims, const fro_sobgrad_params *P, const real *T, const real *S, const real *v0,
                         real lambda, real *grad_v0, double *grad_lambda) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d), N3 = 3 * N;
    const int K = P->iters, Rr = P->width / 2;
    real taps[64];
    FN(gaussian_taps)(P->sigma, P->width, taps);
    /* every state is kept for the reverse sweep; the loss alone needs two */
    const int keep = grad_v0 ? K + 1 : 2;
    real *phis = (real *)malloc(sizeof(real) * N3 * keep);
    real *ms = (real *)malloc(sizeof(real) * N3 * keep);
    real *g = (real *)malloc(sizeof(real) * N3), *tmp = (real *)malloc(sizeof(real) * N3);
    for (int z = 0; z < d.Z; ++z)
        for (int y = 0; y < d.Y; ++y)
            for (int x = 0; x < d.X; ++x) {
                int64_t i = lin(&d, x, y, z);
                phis[i] = (real)x;
                phis[N + i] = (real)y;
                phis[2 * N + i] = (real)z;
            }
    memcpy(ms, v0, sizeof(real) * N3);
    for (int k = 0; k < K; ++k) {
        const int slot = grad_v0 ? k : 0;
        real *phi = phis + (int64_t)slot * N3, *m = ms + (int64_t)slot * N3;
        real *phin = phi + N3, *mn = m + N3;
        FN(sob_grad)(dims, S, T, phi, lambda, g, NULL);
        memcpy(mn, m, sizeof(real) * N3);
        FN(sob_smooth)(dims, taps, Rr, 0, g, tmp, 0, R(0), R(0));
        FN(sob_smooth)(dims, taps, Rr, 1, tmp, g, 0, R(0), R(0));
        FN(sob_smooth)(dims, taps, Rr, 2, g, mn, 1, P->damping, P->step);
        memcpy(phin, phi, sizeof(real) * N3);
        real mx;
        int64_t am;
        FN(sob_pass_b)(dims, mn, phin, &mx, &am);
        if (!grad_v0) {
            memcpy(phi, phin, sizeof(real) * N3);
            memcpy(m, mn, sizeof(real) * N3);
        }
    }
    const int last = grad_v0 ? K : 0;
    const real *phiK = phis + (int64_t)last * N3, *mK = ms + (int64_t)last * N3;
    double J = 0.0;
    real *pbar = grad_v0 ? (real *)calloc(N3, sizeof(real)) : NULL;
    for (int64_t i = 0; i < N; ++i) {
        fro_scell s;
        sob_locate_(&d, phiK[i], phiK[N + i], phiK[2 * N + i], &s);
        fro_tri t;
        tri_eval_(&d, S, &s, &t, 0);
        const real r = t.val - T[i];
        J += 0.5 * (double)r * (double)r;
        if (pbar)
            for (int j = 0; j < 3; ++j) pbar[j * N + i] = r * t.d[j];
    }
    for (int64_t i = 0; i < N3; ++i) J += 0.1 * (double)mK[i] * (double)mK[i];
    if (!grad_v0) {
        free(phis); free(ms); free(g); free(tmp);
        return J;
    }
    real *mbar = (real *)malloc(sizeof(real) * N3);
    for (int64_t i = 0; i < N3; ++i) mbar[i] = R(0.2) * mK[i];
    real *pbar_k = (real *)malloc(sizeof(real) * N3);
    real *gbar = (real *)malloc(sizeof(real) * N3);
    int64_t *cell_base = (int64_t *)malloc(sizeof(int64_t) * N);
    real *cell_w = (real *)malloc(sizeof(real) * 8 * N);
    double *lpart = (double *)malloc(sizeof(double) * d.Z);
    double lbar = 0.0;
    for (int k = K - 1; k >= 0; --k) {
        const real *phi = phis + (int64_t)k * N3, *mn = ms + (int64_t)(k + 1) * N3;
        /* phi_{k+1} = phi_k + m_{k+1}(phi_k): the per-voxel part in parallel (it reads m,
         * which nothing here writes), then the scatter into mbar in voxel order */
        memcpy(pbar_k, pbar, sizeof(real) * N3);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            fro_scell s;
            sob_locate_(&d, phi[i], phi[N + i], phi[2 * N + i], &s);
            for (int c = 0; c < 3; ++c) {
                fro_tri t;
                tri_eval_(&d, mn + c * N, &s, &t, 0);
                const real pb = pbar[c * N + i];
                for (int j = 0; j < 3; ++j) pbar_k[j * N + i] += pb * t.d[j];
                if (c == 0) {
                    cell_base[i] = t.off[0];
                    for (int q = 0; q < 8; ++q) cell_w[8 * i + q] = t.w[q];
                }
            }
        }
        {
            const int64_t X = d.X, XY = (int64_t)d.X * d.Y;
            const int64_t off[8] = {0, 1, X, 1 + X, XY, 1 + XY, X + XY, 1 + X + XY};
            for (int64_t i = 0; i < N; ++i)
                for (int c = 0; c < 3; ++c) {
                    const real pb = pbar[c * N + i];
                    for (int q = 0; q < 8; ++q) mbar[c * N + cell_base[i] + off[q]] += cell_w[8 * i + q] * pb;
                }
        }
        /* m_{k+1} = damping * m_k - step * gs */
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N3; ++i) {
            g[i] = -P->step * mbar[i];
            mbar[i] = P->damping * mbar[i];
        }
        /* gs = Gz Gy Gx g  ->  gbar = Gx^T Gy^T Gz^T gsbar */
        smooth_t_(&d, taps, Rr, 2, g, tmp);
        smooth_t_(&d, taps, Rr, 1, tmp, g);
        smooth_t_(&d, taps, Rr, 0, g, gbar);
        /* g = r dW + lambda lap(u): per voxel, in parallel over slices; dJ/dlambda from
         * per-slice partial sums added in slice order */
#pragma omp parallel for schedule(static)
        for (int z = 0; z < d.Z; ++z) {
            double lz = 0.0;
            for (int y = 0; y < d.Y; ++y)
                for (int x = 0; x < d.X; ++x) {
                    const int64_t i = lin(&d, x, y, z);
                    real lap[3];
                    lap_u_(&d, phi, x, y, z, lap);
                    for (int c = 0; c < 3; ++c) lz += (double)gbar[c * N + i] * (double)lap[c];
                    /* Laplacian part: graph Laplacian is symmetric */
                    const int64_t X = d.X, XY = (int64_t)d.X * d.Y;
                    const int ok[6] = {x > 0, x < d.X - 1, y > 0, y < d.Y - 1, z > 0, z < d.Z - 1};
                    const int64_t off[6] = {-1, 1, -X, X, -XY, XY};
                    for (int c = 0; c < 3; ++c)
                        for (int kk = 0; kk < 6; ++kk)
                            if (ok[kk]) pbar_k[c * N + i] += lambda * (gbar[c * N + i] - gbar[c * N + i + off[kk]]);
                    /* data part: d/dphi of (S(phi) - T) dS(phi) */
                    fro_scell s;
                    sob_locate_(&d, phi[i], phi[N + i], phi[2 * N + i], &s);
                    fro_tri t;
                    tri_eval_(&d, S, &s, &t, 1);
                    const real r = t.val - T[i];
                    real gd = R(0);
                    for (int c = 0; c < 3; ++c) gd += gbar[c * N + i] * t.d[c];
                    for (int j = 0; j < 3; ++j) {
                        real h = R(0);
                        for (int c = 0; c < 3; ++c) h += gbar[c * N + i] * t.H[c][j];
                        pbar_k[j * N + i] += gd * t.d[j] + r * h;
                    }
                }
            lpart[z] = lz;
        }
        for (int z = 0; z < d.Z; ++z) lbar += lpart[z];
        memcpy(pbar, pbar_k, sizeof(real) * N3);
    }
    memcpy(grad_v0, mbar, sizeof(real) * N3);
    *grad_lambda = lbar;
    free(phis); free(ms); free(g); free(tmp); free(pbar); free(mbar); free(pbar_k); free(gbar);
    free(cell_base); free(cell_w); free(lpart);
    return J;
}

/* adjoint of the warp W = img(pos) (sobolev cell): pos_bar = Wbar * dimg/dpos,
 * img_bar(corner) += weight * Wbar */
void FN(warp_adjoint)(const int *dims, const real *pos, const real *img, const real *wbar, real *pos_bar,
                      real *img_bar) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    memset(img_bar, 0, sizeof(real) * N);
    for (int64_t i = 0; i < N; ++i) {
        fro_scell s;
        sob_locate_(&d, pos[i], pos[N + i], pos[2 * N + i], &s);
        fro_tri t;
        tri_eval_(&d, img, &s, &t, 0);
        for (int j = 0; j < 3; ++j) pos_bar[j * N + i] = wbar[i] * t.d[j];
        for (int q = 0; q < 8; ++q) img_bar[t.off[q]] += t.w[q] * wbar[i];
    }
}

/* the warp with the sobolev cell (value only), for finite differences of the adjoint */
void FN(warp_sob)(const int *dims, const real *pos, const real *img, real *out) {
    fro_dims d = {dims[0], dims[1], dims[2]};
    const int64_t N = nvox(&d);
    for (int64_t i = 0; i < N; ++i) {
        fro_scell s;
        sob_locate_(&d, pos[i], pos[N + i], pos[2 * N + i], &s);
        fro_tri t;
        tri_eval_(&d, img, &s, &t, 0);
        out[i] = t.val;
    }
}
