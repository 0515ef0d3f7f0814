// tp_mixed.cuh -- FP32 field evaluation from 64-bit fixed-point positions.
#pragma once
#include "tp_common.cuh"

namespace tp {
namespace mixed {

// Two plane-wave modes A, B in FP32, 80 bytes read as five 16-byte loads:
// per mode the lattice vector n and the phase offset in 32-bit fixed point
// (revolutions * 2^32), then the amplitudes as packed FP32 pairs in the order
// (bA0,bA1) (bA2,eA0) | (eA1,eA2) (bB0,bB1) | (bB2,eB0) (eB1,eB2).  An odd
// mode count is padded with a zero-amplitude mode.
struct alignas(16) ModePair {
    int4 nph[2];
    ulonglong2 amp[3];
};

struct MixField {
    int system_type;
    int bc_flag;
    float cm;
    double min[3], L[3];
    float invL[3];
    // ABC force-free field (src/force_free.c:138-150): B0 (A sin lz + C cos ly, ...)
    float A, Bc, C, B0;
    int abc_fixed;           // lambda * L / 2pi integral on every axis: exact fixed-point phase
    uint32_t abc_m[3];       // lambda * L_k / 2pi
    uint32_t abc_off[3];     // lambda * min_k / 2pi in revolutions * 2^32
    float lam, lmin[3], lL[3];
    // gridded fields: node-interleaved {Ex,Ey,Ez,Bx,By,Bz,0,0} (PIC, 32 bytes a
    // node) or {v,0} (ABC velocity)
    int nx, ny, nz;
    int interp_ref;          // 1: the reference's weights (x and z fractions exchanged)
    const float4* eb;        // two float4 per node
    const float4* vgrid;
    // plane-wave mode sum, B = mB0 z + sum
    int nmodes;
    const ModePair* modes;   // (nmodes + 1) / 2 records
    float mB0;
};

__device__ __forceinline__ float rev_to_rad(uint32_t ph)
{
    return (float)(int32_t)ph * 1.46291807926715968e-9f;  // 2 pi / 2^32
}

// cell index and fraction along one axis from the top 32 bits of a position
__device__ __forceinline__ void cell_of(uint64_t X, int n, int& i, float& fr)
{
    uint64_t G = (X >> 32) * (uint64_t)(uint32_t)(n - 1);
    i = (int)(G >> 32);
    fr = (float)(uint32_t)G * 2.3283064365386963e-10f;  // 2^-32
}

// Packed FP32 pairs (f32x2): two lanes of one 64-bit register, each rounded as
// the scalar operation would be.
__device__ __forceinline__ uint64_t pack_f2(float a, float b)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpack_f2(uint64_t v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t mul_f2(uint64_t a, uint64_t b)
{
    uint64_t r;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t fma_f2(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t r;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// One node {Ex,Ey,Ez,Bx,By,Bz,0,0} (32 bytes, 32-byte aligned) from global
// memory through the read-only path in one 256-bit load, as three packed FP32
// pairs (Ex,Ey) (Ez,Bx) (By,Bz); the padding pair is loaded and dropped.
__device__ __forceinline__ void ld_node32(const float4* p, uint64_t& exy, uint64_t& ezbx, uint64_t& bybz)
{
    uint64_t pad;
    asm volatile("ld.global.nc.v4.b64 {%0,%1,%2,%3}, [%4];"
                 : "=l"(exy), "=l"(ezbx), "=l"(bybz), "=l"(pad)
                 : "l"(p));
}

// The eight corner nodes of the cell a particle last sampled, kept in
// registers: at a few tenths of a cell per step most evaluations fall in the
// same cell as the previous one and need no memory traffic at all.
template <int STRIDE>
struct CellCache {
    uint32_t key = 0xffffffffu;  // node index of the cached cell (grids hold < 2^32 - 1 nodes)
    float4 c[8 * STRIDE];
};

// The same for the gridded E and B: per corner the six components as three
// packed FP32 pairs, 48 registers.
struct CellCacheEB {
    uint32_t key = 0xffffffffu;
    uint64_t c[8][3];
};

// The cell of a position along one axis, with the reference's exchange of the
// x and z fractions (src/interpolation.c:173-180) when interp_ref is set.
__device__ __forceinline__ uint32_t cell_and_weights(const MixField& f, const uint64_t X[3], float w[8])
{
    int ix, iy, iz;
    float fx, fy, fz;
    cell_of(X[0], f.nx, ix, fx);
    cell_of(X[1], f.ny, iy, fy);
    cell_of(X[2], f.nz, iz, fz);
    if (f.interp_ref) {
        float t = fx;
        fx = fz;
        fz = t;
    }
    const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
    const float a00 = gy * gz, a10 = fy * gz, a01 = gy * fz, a11 = fy * fz;
    w[0] = gx * a00; w[1] = fx * a00; w[2] = gx * a10; w[3] = fx * a10;
    w[4] = gx * a01; w[5] = fx * a01; w[6] = gx * a11; w[7] = fx * a11;
    return (uint32_t)ix + (uint32_t)f.nx * iy + (uint32_t)f.nx * f.ny * iz;
}

// Trilinear E and B from the node-interleaved grid: the eight corner weights
// once, then per pair of components one multiply and seven packed FMAs, in
// corner order (each component's products and sums are those of a scalar
// loop).
__device__ __forceinline__ void trilinear_eb(const MixField& f, const uint64_t X[3], CellCacheEB& cc,
                                             float E[3], float B[3])
{
    float w[8];
    const uint32_t base = cell_and_weights(f, X, w);
    if (base != cc.key) {
        const uint32_t nx = f.nx, nxy = (uint32_t)f.nx * f.ny;
        const float4* p = f.eb + (size_t)base * 2;
        const uint32_t off[8] = {0, 1, nx, nx + 1, nxy, nxy + 1, nxy + nx, nxy + nx + 1};
#pragma unroll
        for (int k = 0; k < 8; k++) ld_node32(p + (size_t)off[k] * 2, cc.c[k][0], cc.c[k][1], cc.c[k][2]);
        cc.key = base;
    }
    uint64_t wp = pack_f2(w[0], w[0]);
    uint64_t r0 = mul_f2(wp, cc.c[0][0]), r1 = mul_f2(wp, cc.c[0][1]), r2 = mul_f2(wp, cc.c[0][2]);
#pragma unroll
    for (int k = 1; k < 8; k++) {
        wp = pack_f2(w[k], w[k]);
        r0 = fma_f2(wp, cc.c[k][0], r0);
        r1 = fma_f2(wp, cc.c[k][1], r1);
        r2 = fma_f2(wp, cc.c[k][2], r2);
    }
    unpack_f2(r0, E[0], E[1]);
    unpack_f2(r1, E[2], B[0]);
    unpack_f2(r2, B[1], B[2]);
}

// trilinear interpolation of a node-interleaved field with `stride` float4s per node
template <int STRIDE>
__device__ __forceinline__ void trilinear_f(const MixField& f, const float4* __restrict__ g,
                                            const uint64_t X[3], CellCache<STRIDE>& cc,
                                            float4 out[STRIDE])
{
    int ix, iy, iz;
    float fx, fy, fz;
    cell_of(X[0], f.nx, ix, fx);
    cell_of(X[1], f.ny, iy, fy);
    cell_of(X[2], f.nz, iz, fz);
    if (f.interp_ref) {  // src/interpolation.c:173-180 pairs x weights with z corners
        float t = fx;
        fx = fz;
        fz = t;
    }
    const uint32_t nx = f.nx, nxy = (uint32_t)f.nx * f.ny;
    const uint32_t base = ix + nx * iy + nxy * iz;
    if (base != cc.key) {
        const float4* p = g + (size_t)base * STRIDE;
#pragma unroll
        for (int c = 0; c < STRIDE; c++) {
            cc.c[0 * STRIDE + c] = __ldg(p + c);
            cc.c[1 * STRIDE + c] = __ldg(p + STRIDE + c);
            cc.c[2 * STRIDE + c] = __ldg(p + nx * STRIDE + c);
            cc.c[3 * STRIDE + c] = __ldg(p + (nx + 1) * STRIDE + c);
            cc.c[4 * STRIDE + c] = __ldg(p + nxy * STRIDE + c);
            cc.c[5 * STRIDE + c] = __ldg(p + (nxy + 1) * STRIDE + c);
            cc.c[6 * STRIDE + c] = __ldg(p + (nxy + nx) * STRIDE + c);
            cc.c[7 * STRIDE + c] = __ldg(p + (nxy + nx + 1) * STRIDE + c);
        }
        cc.key = base;
    }
    // eight corner weights once, then one multiply and seven FMAs per component
    const float gx = 1.0f - fx, gy = 1.0f - fy, gz = 1.0f - fz;
    const float a00 = gy * gz, a10 = fy * gz, a01 = gy * fz, a11 = fy * fz;
    const float w[8] = {gx * a00, fx * a00, gx * a10, fx * a10, gx * a01, fx * a01, gx * a11, fx * a11};
#pragma unroll
    for (int c = 0; c < STRIDE; c++) {
        // packed FP32 pairs (x, y) and (z, pad): the same products and sums,
        // in the same order, with half the instructions
        uint64_t wp = pack_f2(w[0], w[0]);
        uint64_t rxy = mul_f2(wp, pack_f2(cc.c[c].x, cc.c[c].y));
        uint64_t rzw = mul_f2(wp, pack_f2(cc.c[c].z, cc.c[c].w));
#pragma unroll
        for (int k = 1; k < 8; k++) {
            const float4 v = cc.c[k * STRIDE + c];
            wp = pack_f2(w[k], w[k]);
            rxy = fma_f2(wp, pack_f2(v.x, v.y), rxy);
            rzw = fma_f2(wp, pack_f2(v.z, v.w), rzw);
        }
        float4 r;
        unpack_f2(rxy, r.x, r.y);
        unpack_f2(rzw, r.z, r.w);
        r.w = 0.f;
        out[c] = r;
    }
}

// Per-particle register state of the field evaluation.
struct FieldCache {
    CellCacheEB eb;    // gridded E, B
    CellCache<1> v;    // ABC velocity grid
};

template <int SYS>
__device__ __forceinline__ void field_mixed(const MixField& f, const uint64_t X[3], float E[3],
                                            float B[3], const ModePair* smodes, FieldCache& fc)
{
    E[0] = E[1] = E[2] = 0.f;
    if (SYS == TP_SYS_TEST) {
        B[0] = 0.f; B[1] = 0.f; B[2] = 1.0f;
    } else if (SYS == TP_SYS_FORCEFREE) {
        float sx, cx, sy, cy, sz, cz;
        if (f.abc_fixed) {
            __sincosf(rev_to_rad((uint32_t)(X[0] >> 32) * f.abc_m[0] + f.abc_off[0]), &sx, &cx);
            __sincosf(rev_to_rad((uint32_t)(X[1] >> 32) * f.abc_m[1] + f.abc_off[1]), &sy, &cy);
            __sincosf(rev_to_rad((uint32_t)(X[2] >> 32) * f.abc_m[2] + f.abc_off[2]), &sz, &cz);
        } else {
            sincosf(f.lmin[0] + f.lL[0] * ((float)(X[0] >> 40) * 5.9604644775390625e-8f), &sx, &cx);
            sincosf(f.lmin[1] + f.lL[1] * ((float)(X[1] >> 40) * 5.9604644775390625e-8f), &sy, &cy);
            sincosf(f.lmin[2] + f.lL[2] * ((float)(X[2] >> 40) * 5.9604644775390625e-8f), &sz, &cz);
        }
        B[0] = f.B0 * (f.A * sz + f.C * cy);
        B[1] = f.B0 * (f.Bc * sx + f.A * cz);
        B[2] = f.B0 * (f.C * sy + f.Bc * cx);
        if (f.vgrid) {  // E = -v x B, src/force_free.c:78-86
            float4 v;
            trilinear_f<1>(f, f.vgrid, X, fc.v, &v);
            E[0] = B[1] * v.z - B[2] * v.y;
            E[1] = B[2] * v.x - B[0] * v.z;
            E[2] = B[0] * v.y - B[1] * v.x;
        }
    } else if (SYS == TP_SYS_PIC) {
        trilinear_eb(f, X, fc.eb, E, B);
    } else if (SYS == TP_SYS_MODESUM) {
        const uint32_t X32 = (uint32_t)(X[0] >> 32), Y32 = (uint32_t)(X[1] >> 32),
                       Z32 = (uint32_t)(X[2] >> 32);
        // accumulators (b0,b1) (b2,e0) (e1,e2); each lane sums the modes in
        // table order with one FMA per mode, as a scalar loop would
        uint64_t s01 = 0, s23 = 0, s45 = 0;
        const int npairs = (f.nmodes + 1) >> 1;
#pragma unroll 2
        for (int q = 0; q < npairs; q++) {
            const int4 na = smodes[q].nph[0], nb = smodes[q].nph[1];
            const ulonglong2 w0 = smodes[q].amp[0], w1 = smodes[q].amp[1], w2 = smodes[q].amp[2];
            const uint32_t pa = (uint32_t)na.x * X32 + (uint32_t)na.y * Y32 + (uint32_t)na.z * Z32 + (uint32_t)na.w;
            const uint32_t pb = (uint32_t)nb.x * X32 + (uint32_t)nb.y * Y32 + (uint32_t)nb.z * Z32 + (uint32_t)nb.w;
            const float ca = __cosf(rev_to_rad(pa)), cb = __cosf(rev_to_rad(pb));
            const uint64_t cca = pack_f2(ca, ca), ccb = pack_f2(cb, cb);
            s01 = fma_f2(w0.x, cca, s01); s23 = fma_f2(w0.y, cca, s23); s45 = fma_f2(w1.x, cca, s45);
            s01 = fma_f2(w1.y, ccb, s01); s23 = fma_f2(w2.x, ccb, s23); s45 = fma_f2(w2.y, ccb, s45);
        }
        float b2;
        unpack_f2(s01, B[0], B[1]);
        unpack_f2(s23, b2, E[0]);
        unpack_f2(s45, E[1], E[2]);
        B[2] = f.mB0 + b2;
    }
}

}  // namespace mixed
}  // namespace tp
