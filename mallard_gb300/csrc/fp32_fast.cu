// fp32_fast.cu -- the FP32-bulk form of the reconstruction and face flux.
//
// Arithmetic split (everything else stays FP64):
//  * FP32: TENO coefficients, smoothness indicators, stencil selection, face
//    evaluation, face states, primitive recovery, Riemann flux, viscous
//    terms (and, in spectral32.cuh, the time step's spectral radius);
//  * FP64: the table build (least squares, face shapes; the tables are
//    rounded to FP32 once, on upload), geometry (normals, areas, volumes),
//    the conserved state and its accumulation across RK stages in the
//    update kernel (which also writes an FP32 copy of each stage's state for
//    the reconstruction to gather), and primitive recovery near vacuum: when
//    the internal energy is under 1e-3 of the total the face state is
//    recovered in FP64.
// Stencil selection uses ratios of smoothness indicators: (SI+eps)^-6 itself
// overflows FP32, but w_s / sum w = 1 / sum_d ((SI_s+eps)/(SI_d+eps))^6 does
// not.  Only the corrected weighting is built in this form.
#include <algorithm>
#include <cstdint>

#include "fp_convert.cuh"
#include "physics.cuh"

namespace mgpu {
namespace f32 {
namespace {

// FP64 -> FP32 of the state gathered from the FP64 stage arrays and of the
// FP64 constants: round to nearest on the integer pipe (fp_convert.cuh).
__device__ __forceinline__ float f(double x) { return f32_rn(x); }

// SEL: per (cell, variable) predictions of the learned selector (pred:
// predicted mask, bit 7 = confident).  A confident variable takes the
// predicted stencils with equal weights and computes no smoothness
// indicator; a cell evaluates only the stencils that one of its variables
// needs, all of them as soon as one variable is not confident.
// Row indices of state and face arrays.  Ix1: one case, rows in the mesh's
// own order.  IxB: case cs of a batch group of C cases sharing one mesh,
// rows interleaved per 8-row tile: row(c) = base + ((c / 8) C + cs) 8 + c % 8.
struct Ix1 {
    __device__ __forceinline__ size_t u(size_t c) const { return c; }
    __device__ __forceinline__ size_t f(size_t fi) const { return fi; }
};
struct IxB {
    size_t ubase, fbase;
    unsigned C, cs;
    __device__ __forceinline__ size_t u(size_t c) const { return ubase + (((c >> 3) * C + cs) << 3) + (c & 7); }
    __device__ __forceinline__ size_t f(size_t fi) const { return fbase + (((fi >> 3) * C + cs) << 3) + (fi & 7); }
};

// Table blocks of one tile: for stencil s the neighbour ids [GJ][8] uint4
// and the pseudo-inverse [GP][8] float4, and the face-shape codes of its 8
// cells (16 bytes), each contiguous in the tiled arrays.
template <int K, int M, int NQ>
struct TileBlocks {
    static constexpr int KR = K - 1, MR = M - 1, NF = 3, S = 4;
    static constexpr int GJ = (MR + 3) / 4, GP = (MR * KR + 3) / 4;
    static constexpr int GT = (NQ * KR + 3) / 4;  // float4 per shape set of the code table
    static constexpr unsigned PB = GP * TILE * 16, NBB = GJ * TILE * 16, CB = TILE * 2;
    static_assert(CB == 16, "one 16-byte bulk copy of a tile's codes");
};

// Table source of teno32_cell: the tiled arrays in global memory.
template <int K, int M, int NQ>
struct GlobalSrc {
    using B = TileBlocks<K, M, NQ>;
    const TenoArgs& a;
    int tile;
    __device__ __forceinline__ unsigned tile_need(unsigned need) const { return need; }
    __device__ __forceinline__ bool begin(int) { return true; }
    __device__ __forceinline__ void end(int) {}
    __device__ __forceinline__ const uint4* nb(int s) const {
        return reinterpret_cast<const uint4*>(a.nb4) + (size_t)(tile * B::S + s) * B::GJ * TILE;
    }
    __device__ __forceinline__ const float4* P(int s) const {
        return reinterpret_cast<const float4*>(a.P4) + (size_t)(tile * B::S + s) * B::GP * TILE;
    }
    __device__ __forceinline__ const uint16_t* codes() { return a.fcode + (size_t)tile * TILE; }
    template <class T>
    __device__ __forceinline__ T ld(const T* p) const { return __ldg(p); }
};

// (u, v, T) of an FP32 state with one correctly rounded reciprocal of the
// density.
__device__ __forceinline__ float4 uvT32(const float4 x, float inv_cv) {
    const float ir = __frcp_rn(x.x);
    const float u = x.y * ir, v = x.z * ir;
    const float e = x.w * ir - 0.5f * (u * u + v * v);
    return make_float4(u, v, e * inv_cv, 0.0f);
}

// The robust variant's per-cell step in FP32 (teno_flux.cuh's robust_cell):
// a cell with a boundary face takes its average at every face point;
// otherwise each variable's deviations are scaled into the central
// stencil's range [dlo, dhi] (when that stencil was evaluated), and a cell
// with a face state that is then not admissible takes its average at every
// face point.  Every lane of live calls it (the cell's four lanes exchange
// their variables).  Returns the factor the variable's polynomial was
// scaled by (1: kept, 0: replaced by the average).
template <int NF, int NQ>
__device__ __forceinline__ float robust_cell32(const TenoArgs& a, bool boundary, bool have_range, unsigned live,
                                               float uc, float dlo, float dhi, float (&out)[NF][NQ]) {
    float th = 1.0f;
    if (!boundary && have_range) {
#pragma unroll
        for (int fl = 0; fl < NF; ++fl)
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const float d = out[fl][q] - uc;
                if (d > dhi) th = fminf(th, dhi / d);
                else if (d < dlo) th = fminf(th, dlo / d);
            }
        if (th < 1.0f)
#pragma unroll
            for (int fl = 0; fl < NF; ++fl)
#pragma unroll
                for (int q = 0; q < NQ; ++q) out[fl][q] = fmaf(th, out[fl][q] - uc, uc);
    }
    bool bad = boundary;
#pragma unroll
    for (int fl = 0; fl < NF; ++fl)
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const float rho = __shfl_sync(live, out[fl][q], 0, 4);
            const float m0 = __shfl_sync(live, out[fl][q], 1, 4);
            const float m1 = __shfl_sync(live, out[fl][q], 2, 4);
            const float E = __shfl_sync(live, out[fl][q], 3, 4);
            const float m2 = fmaf(m0, m0, m1 * m1);
            if (!(rho > 0.0f && 2.0f * rho * E > m2)) bad = true;
        }
    if (bad)
#pragma unroll
        for (int fl = 0; fl < NF; ++fl)
#pragma unroll
            for (int q = 0; q < NQ; ++q) out[fl][q] = uc;
    return bad ? 0.0f : th;
}

// Viscous gradients from the reconstruction in FP32 (teno_flux.cuh's
// write_visc_grad): lane v holds the gradient (gx, gy) of conserved
// variable v's polynomial at the cell centroid and the cell average uc;
// lane 0 of the cell writes the Visc32Args records when `write`.  Every lane
// of live calls it.
__device__ __forceinline__ void write_visc_grad32(const TenoArgs& a, int cell, int v, unsigned live, float uc,
                                                  float gx, float gy, bool write) {
    float r[4], x[4], y[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        r[i] = __shfl_sync(live, uc, i, 4);
        x[i] = __shfl_sync(live, gx, i, 4);
        y[i] = __shfl_sync(live, gy, i, 4);
    }
    if (v != 0 || !write) return;
    const float4 q = uvT32(make_float4(r[0], r[1], r[2], r[3]), a.inv_cv);
    const float ir = __frcp_rn(r[0]), E = r[3] * ir;
    const float ux = (x[1] - q.x * x[0]) * ir, uy = (y[1] - q.x * y[0]) * ir;
    const float vx = (x[2] - q.y * x[0]) * ir, vy = (y[2] - q.y * y[0]) * ir;
    const float ex = (x[3] - E * x[0]) * ir - fmaf(q.x, ux, q.y * vx);
    const float ey = (y[3] - E * y[0]) * ir - fmaf(q.x, uy, q.y * vy);
    a.vq[cell] = q;
    a.vga[cell] = make_float4(ux, uy, vx, vy);
    a.vgb[cell] = make_float2(ex * a.inv_cv, ey * a.inv_cv);
}

// Reconstruction of variable v of one cell.  live: lanes of the warp whose
// cells exist (the four lanes of a cell share its fate).  src: where the
// tile's table blocks are read (GlobalSrc, or shared memory filled by bulk
// copies); the stencil loop visits src.tile_need(need), which a shared-memory
// source makes the same for the whole warp.  Returns false when the source
// failed (nothing written).  alive false: a lane past the mesh that only
// takes part in the warp's collective steps (reads and writes nothing).
template <int K, int M, int NQ, bool SEL, bool VG, class IX, class SRC>
__device__ __forceinline__ bool teno32_cell(const TenoArgs& a, const float* __restrict__ U, float* __restrict__ fv,
                                            uint8_t* __restrict__ masks, const uint8_t* __restrict__ pred, int cell,
                                            int v, unsigned live, const IX& ix, SRC& src, bool alive = true) {
    constexpr int KR = K - 1, MR = M - 1, NF = 3, S = 4;
    constexpr int GJ = (MR + 3) / 4, GP = (MR * KR + 3) / 4, GT = (NQ * KR + 3) / 4;
    const int tile = cell >> 3, lane = cell & 7;
    const float uc = alive ? U[ix.u(cell) * NC + v] : 0.0f;
    const unsigned sm = alive ? a.smask[cell] : 0u;
    unsigned need = sm, pm = 0;
    bool conf = false;
    if (SEL) {
        const unsigned p = alive ? pred[ix.u(cell) * NC + v] : 0u;
        pm = p & sm & 0xFu;
        conf = (p & 0x80u) && pm;
        unsigned my = conf ? pm : sm;
        my |= __shfl_xor_sync(live, my, 1);
        my |= __shfl_xor_sync(live, my, 2);
        need = my;
    }

    const unsigned tile_need = src.tile_need(need);
    bool ok = true;
    float coef[S][KR];
    float x[S];
    float dlo = 0.0f, dhi = 0.0f;  // robust variant: central-stencil range around uc
    bool have_range = false;
#pragma unroll
    for (int s = 0; s < S; ++s) {
#pragma unroll
        for (int k = 0; k < KR; ++k) coef[s][k] = 0.0f;
        x[s] = 0.0f;
        if (!((tile_need >> s) & 1u)) continue;
        ok = src.begin(s) && ok;
        if (ok && ((need >> s) & 1u)) {
            // differences to the target cell's average over the stencil
            const uint4* nbp = src.nb(s) + lane;
            float d[GJ * 4];
#pragma unroll
            for (int g = 0; g < GJ; ++g) {
                const uint4 n = src.ld(nbp + g * TILE);
                const uint32_t id[4] = {n.x, n.y, n.z, n.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (g * 4 + e < MR) d[g * 4 + e] = __ldg(U + ix.u(id[e]) * NC + v) - uc;
            }
            if (s == 0 && a.bcell) {
#pragma unroll
                for (int j = 0; j < MR; ++j) {
                    dlo = fminf(dlo, d[j]);
                    dhi = fmaxf(dhi, d[j]);
                }
                have_range = true;
            }
            // coefficients = (P x areas) . d, accumulated over the stencil in order
            const float4* Pp = src.P(s) + lane;
#pragma unroll
            for (int g = 0; g < GP; ++g) {
                const float4 p4 = src.ld(Pp + g * TILE);
                const float pv[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int fl = g * 4 + e;
                    if (fl < MR * KR) coef[s][fl % KR] = fmaf(pv[e], d[fl / KR], coef[s][fl % KR]);
                }
            }
            if (!(SEL && conf)) {
                float si = 0.0f;
#pragma unroll
                for (int i = 0; i < KR; ++i) {
                    float oa = a.oi2f[i * KR + i] * coef[s][i];
#pragma unroll
                    for (int l = i + 1; l < KR; ++l) oa = fmaf(a.oi2f[i * KR + l], coef[s][l], oa);
                    si = fmaf(coef[s][i], oa, si);
                }
                x[s] = si + 1.0e-12f;
            }
        }
        src.end(s);
    }

    unsigned mask = 0;
    float w[S] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (SEL && conf) {
        mask = pm;
        if (pm & 1u) {
            w[0] = 1.0f;
        } else {
            const float share = 1.0f / (float)__popc(pm);
#pragma unroll
            for (int s = 1; s < S; ++s) w[s] = ((pm >> s) & 1u) ? share : 0.0f;
        }
    } else {
    // stencil selection in ratio form
    float rx[S];
#pragma unroll
    for (int s = 1; s < S; ++s) rx[s] = ((sm >> s) & 1u) ? 1.0f / x[s] : 0.0f;
    float r = 0.0f;
#pragma unroll
    for (int d = 1; d < S; ++d) {
        const float q = x[0] * rx[d], q2 = q * q;
        r = fmaf(q2 * q2, q2, r);
    }
    if (r < 9999999.0f) {  // w0 / (w0 + sum_d w_d) > 1e-7
        mask = 1;
        w[0] = 1.0f;
    } else {
        int npass = 0;
#pragma unroll
        for (int s = 1; s < S; ++s) {
            if (!((sm >> s) & 1u)) continue;
            float t = 0.0f;
#pragma unroll
            for (int d = 1; d < S; ++d) {
                const float q = x[s] * rx[d], q2 = q * q;
                t = fmaf(q2 * q2, q2, t);
            }
            if (t < 1.0e5f) {  // w_s / sum_d w_d > 1e-5
                mask |= 1u << s;
                ++npass;
            }
        }
        const float share = npass ? 1.0f / (float)npass : 0.0f;
#pragma unroll
        for (int s = 1; s < S; ++s) w[s] = ((mask >> s) & 1u) ? share : 0.0f;
    }
    }
    if (ok && alive && masks) masks[ix.u(cell) * NC + v] = (uint8_t)mask;
    // blended coefficients
    float c[KR];
#pragma unroll
    for (int k = 0; k < KR; ++k) {
        float t = 0.0f;
#pragma unroll
        for (int s = 0; s < S; ++s) t = fmaf(coef[s][k], w[s], t);
        c[k] = t;
    }

    // face values: the shapes of each face slot's code (a 3-bit index into
    // the shared table: always in bounds), then one dot product per point.
    // The robust variant's per-cell step needs every lane of the live mask
    // (its four lanes per cell exchange their variables), so a lane with
    // nothing to write still computes (on code 0) and takes part.
    const uint16_t* codes = src.codes();
    const bool fine = codes && ok && alive;
    const bool robust = a.bcell != nullptr;
    const bool vgrad = VG && a.vq != nullptr;  // single-case layout (Ix1) only
    if (!fine && !robust && !vgrad) return false;
    const unsigned code = fine ? src.ld(codes + lane) : 0u;
    float outv[NF][NQ];
    uint32_t slots[NF];
#pragma unroll
    for (int fl = 0; fl < NF; ++fl) {
        slots[fl] = fine ? __ldg(a.cface + ((size_t)tile * NF + fl) * TILE + lane) : 0u;
        const float4* t4 = a.phi_tab4 + ((code >> (3 * fl)) & 7u) * GT;
        float phi[GT * 4];
#pragma unroll
        for (int g = 0; g < GT; ++g) {
            const float4 p4 = __ldg(t4 + g);
            phi[g * 4] = p4.x;
            phi[g * 4 + 1] = p4.y;
            phi[g * 4 + 2] = p4.z;
            phi[g * 4 + 3] = p4.w;
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            float out = uc;
#pragma unroll
            for (int k = 0; k < KR; ++k) out = fmaf(c[k], phi[q * KR + k], out);
            outv[fl][q] = out;
        }
    }
    // the polynomial's gradient at the centroid (d/dxi, then the frame's
    // inverse Jacobian)
    float gx = 0.0f, gy = 0.0f;
    if (vgrad) {
        float g0 = 0.0f, g1 = 0.0f;
#pragma unroll
        for (int k = 0; k < KR; ++k) {
            g0 = fmaf(c[k], a.dphif[2 * k], g0);
            g1 = fmaf(c[k], a.dphif[2 * k + 1], g1);
        }
        const float4 J = fine ? __ldg(a.ji4 + cell) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        gx = fmaf(J.x, g0, J.z * g1);
        gy = fmaf(J.y, g0, J.w * g1);
    }
    if (robust) {
        const float keep = robust_cell32<NF, NQ>(a, fine && a.bcell[cell] != 0, have_range, live, uc, dlo, dhi, outv);
        if (keep == 0.0f) {
            gx = 0.0f;
            gy = 0.0f;
        } else if (keep < 1.0f) {
            gx *= keep;
            gy *= keep;
        }
    }
    if (vgrad) write_visc_grad32(a, cell, v, live, uc, gx, gy, fine);
    if (!fine) return false;
#pragma unroll
    for (int fl = 0; fl < NF; ++fl) {
        const size_t fi = slots[fl] >> 1;
        const unsigned side = slots[fl] & 1u;
#pragma unroll
        for (int q = 0; q < NQ; ++q) fv[((ix.f(fi) * NQ + q) * 2 + side) * NC + v] = outv[fl][q];
    }
    return true;
}

template <int K, int M, int NQ, bool SEL, int BS, int MINB, bool VG>
__global__ void __launch_bounds__(BS, MINB) teno32_kernel(const TenoArgs a, const float* __restrict__ U,
                                                          float* __restrict__ fv, uint8_t* __restrict__ masks,
                                                          const uint8_t* __restrict__ pred) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int cell = gt >> 2, v = gt & 3;
    const unsigned live = __ballot_sync(0xffffffffu, cell < a.n_cells);
    if (cell >= a.n_cells) return;
    GlobalSrc<K, M, NQ> src{a, cell >> 3};
    teno32_cell<K, M, NQ, SEL, VG>(a, U, fv, masks, pred, cell, v, live, Ix1{}, src);
}

// Staged form: each warp (one 8-cell tile) copies the table blocks of the
// stencils its cells evaluate into shared memory with cp.async.bulk, NSLOT
// stencils at a time (a slot is refilled with the next stencil as soon as
// the warp is done with it), and the tile's face-shape codes (16 bytes)
// into a slot of their own;
// an mbarrier per slot tracks the bytes.  One bulk copy replaces the dozens
// of dependent table loads of the direct form, so the warp's table traffic
// is in flight at once while it gathers the neighbours' states.
constexpr unsigned STAGE_WAIT_LIMIT = 1u << 22;

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t addr = su32(bar);
    for (unsigned i = 0; i < STAGE_WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}

template <int K, int M, int NQ, int NSLOT>
struct StageLayout {
    using B = TileBlocks<K, M, NQ>;
    static constexpr unsigned SLOT = B::PB + B::NBB;                // pseudo-inverse, then neighbour ids
    static constexpr unsigned PHI = NSLOT * SLOT;                   // face-shape codes of the tile
    static constexpr unsigned BAR = PHI + B::CB;                    // NSLOT + 1 mbarriers
    static constexpr unsigned WARP = (BAR + 8 * (NSLOT + 1) + 127) / 128 * 128;
    static_assert(B::PB % 128 == 0 && B::NBB % 16 == 0 && SLOT % 128 == 0 && B::CB % 16 == 0, "alignment");
};

// Table source of teno32_cell: one warp's shared-memory stage.
template <int K, int M, int NQ, int NSLOT>
struct StageSrc {
    using B = TileBlocks<K, M, NQ>;
    using L = StageLayout<K, M, NQ, NSLOT>;
    const TenoArgs& a;
    uint8_t* base;
    int tile, lane32;
    unsigned need_all = 0;  // stencils some cell of the tile evaluates
    int cnt = 0, issued = 0;
    bool phi_ready = false, ok = true, pre = false;
    __device__ __forceinline__ uint64_t* bar(int i) { return reinterpret_cast<uint64_t*>(base + L::BAR) + i; }
    // the i-th stencil of need_all into slot i % NSLOT (lane 0)
    __device__ __forceinline__ void issue(int i) {
        unsigned m = need_all;
        for (int k = 0; k < i; ++k) m &= m - 1;
        const int s = __ffs(m) - 1;
        uint8_t* slot = base + (i % NSLOT) * L::SLOT;
        mbar_expect_tx(bar(i % NSLOT), L::SLOT);
        bulk_g2s(slot, reinterpret_cast<const char*>(a.P4) + (size_t)(tile * B::S + s) * B::PB, B::PB, bar(i % NSLOT));
        bulk_g2s(slot + B::PB, reinterpret_cast<const char*>(a.nb4) + (size_t)(tile * B::S + s) * B::NBB, B::NBB,
                 bar(i % NSLOT));
    }
    // all lanes, at the warp's start: the central stencil's copy, before
    // the cells' states and predictions (which decide the rest) arrive.
    // The central stencil is then staged for every tile, also one whose
    // cells all skip it (only a confident directional prediction does).
    __device__ __forceinline__ void prefetch_central() {
        need_all = 1u;
        pre = true;
        if (lane32 == 0) issue(0);
    }
    // all lanes: the union of the cells' stencils, then the first copies
    __device__ __forceinline__ unsigned tile_need(unsigned need) {
        need_all = __reduce_or_sync(0xffffffffu, need) | (pre ? 1u : 0u);
        cnt = __popc(need_all);
        issued = cnt < NSLOT ? cnt : NSLOT;
        if (lane32 == 0)
            for (int i = pre ? 1 : 0; i < issued; ++i) issue(i);
        return need_all;
    }
    __device__ __forceinline__ int index(int s) const { return __popc(need_all & ((1u << s) - 1u)); }
    __device__ __forceinline__ bool begin(int s) {
        const int i = index(s);
        const bool done = mbar_wait(bar(i % NSLOT), (unsigned)(i / NSLOT) & 1u);
        ok = __all_sync(0xffffffffu, done) && ok;
        return ok;
    }
    __device__ __forceinline__ void end(int s) {
        const int i = index(s);
        __syncwarp();
        // refill the slot with the next stencil, unless a wait failed
        if (ok && i + NSLOT < cnt) {
            if (lane32 == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(i + NSLOT);
            }
            issued = i + NSLOT + 1;
        }
    }
    __device__ __forceinline__ const uint4* nb(int s) const {
        return reinterpret_cast<const uint4*>(base + (index(s) % NSLOT) * L::SLOT + B::PB);
    }
    __device__ __forceinline__ const float4* P(int s) const {
        return reinterpret_cast<const float4*>(base + (index(s) % NSLOT) * L::SLOT);
    }
    __device__ __forceinline__ const uint16_t* codes() {
        if (!phi_ready) {
            const bool done = mbar_wait(bar(NSLOT), 0u);
            ok = __all_sync(0xffffffffu, done) && ok;
            phi_ready = true;
        }
        return ok ? reinterpret_cast<const uint16_t*>(base + L::PHI) : nullptr;
    }
    template <class T>
    __device__ __forceinline__ T ld(const T* p) const { return *p; }
};

template <int K, int M, int NQ, bool SEL, int NSLOT, int WARPS, int MINB, bool VG>
__global__ void __launch_bounds__(WARPS * 32, MINB) teno32_staged_kernel(const TenoArgs a, const float* __restrict__ U,
                                                                         float* __restrict__ fv,
                                                                         uint8_t* __restrict__ masks,
                                                                         const uint8_t* __restrict__ pred,
                                                                         unsigned* __restrict__ err) {
    using L = StageLayout<K, M, NQ, NSLOT>;
    using B = TileBlocks<K, M, NQ>;
    extern __shared__ __align__(128) uint8_t stage_smem[];
    const int w = threadIdx.x >> 5, lane32 = threadIdx.x & 31;
    const int tile = blockIdx.x * WARPS + w;
    const int n_tiles = (a.n_cells + 7) >> 3;
    if (tile >= n_tiles) return;
    StageSrc<K, M, NQ, NSLOT> src{a, stage_smem + (size_t)w * L::WARP, tile, lane32};
    if (lane32 == 0) {
        for (int i = 0; i <= NSLOT; ++i) mbar_init(src.bar(i), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // the face-shape codes first: needed last, by every cell
        mbar_expect_tx(src.bar(NSLOT), B::CB);
        bulk_g2s(src.base + L::PHI, reinterpret_cast<const char*>(a.fcode) + (size_t)tile * B::CB, B::CB, src.bar(NSLOT));
    }
    __syncwarp();
    src.prefetch_central();
    const int cell = tile * 8 + (lane32 >> 2), v = lane32 & 3;
    // cells past the mesh take part in the warp's collective steps with
    // nothing to do: smask 0, no prediction, no writes
    teno32_cell<K, M, NQ, SEL, VG>(a, U, fv, masks, pred, cell, v, 0xffffffffu, Ix1{}, src, cell < a.n_cells);
    if (!src.ok) {
        // a wait ran out: flag it and give every copy still pending on this
        // warp's stage one more bounded wait before the shared memory goes
        if (lane32 == 0 && err) atomicOr(err, 1u);
        for (int i = 0; i <= NSLOT; ++i) {
            const int uses = i == NSLOT ? 1 : (i < src.issued ? (src.issued - i + NSLOT - 1) / NSLOT : 0);
            if (uses > 0) mbar_wait(src.bar(i), (unsigned)(uses - 1) & 1u);
        }
    }
}

// Primitive recovery of a face state in FP32 with one correctly rounded
// reciprocal of the density (instead of five divisions), or in FP64 when
// the internal energy is a small remainder of the total (near vacuum
// pressure).
__device__ __forceinline__ void primitives_guarded(const GasParams& g, const float* U, float* W) {
    const float rho = U[0], ir = __frcp_rn(rho);
    const float u0 = U[1] * ir, u1 = U[2] * ir;
    const float E = U[3] * ir;
    const float e = E - 0.5f * (u0 * u0 + u1 * u1);
    const float p = fmaxf(g.p_min_f, fminf(g.p_max_f, g.gm1_f * rho * e));
    W[0] = u0;
    W[1] = u1;
    W[2] = p;
    W[3] = e * g.icv_f;
    W[4] = e + p * ir;
    if (!(e > 1.0e-3f * E)) {
        const double Ud[4] = {U[0], U[1], U[2], U[3]};
        double Wd[5];
        primitives(g, Ud, Wd);
#pragma unroll
        for (int i = 0; i < NPR; ++i) W[i] = __double2float_rn(Wd[i]);
    }
}

// ---------------------------------------------------------------------------
// Viscous flux, FP32 form (the FP64 kernels in kernels.cu define it; the
// same operations in FP32 here)
// ---------------------------------------------------------------------------


__global__ void __launch_bounds__(256) visc_grad32_kernel(const Visc32Args a, const BcTable bct,
                                                          const float* __restrict__ U) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const float4* U4 = reinterpret_cast<const float4*>(U);
    const float4 qc = uvT32(U4[c], a.inv_cv);
    float gx[3] = {0.0f, 0.0f, 0.0f}, gy[3] = {0.0f, 0.0f, 0.0f};
    const int4 cf = a.cfaces[c];
    const int ent[4] = {cf.x, cf.y, cf.z, cf.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        if (ent[e] < 0) break;
        const int fi = ent[e];
        const int2 lr = a.lr[fi];
        const float4 gg = a.fgeo[fi];
        const float A = a.fgeo2[fi].x;
        const float sA = lr.x == c ? A : -A;
        float qf[3];
        if (lr.y >= 0) {
            const float4 qo = uvT32(U4[lr.x == c ? lr.y : lr.x], a.inv_cv);
            qf[0] = 0.5f * (qc.x + qo.x);
            qf[1] = 0.5f * (qc.y + qo.y);
            qf[2] = 0.5f * (qc.z + qo.z);
        } else {
            const int bi = a.bc[fi];
            const bool wall = bi >= 0 && bct.bc[bi].type == MGPU_BC_WALL_ADIABATIC;
            qf[0] = wall ? 0.0f : qc.x;
            qf[1] = wall ? 0.0f : qc.y;
            qf[2] = qc.z;
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            gx[k] = fmaf(qf[k], gg.x * sA, gx[k]);
            gy[k] = fmaf(qf[k], gg.y * sA, gy[k]);
        }
    }
    const float iv = f(a.ivol[c]);
    a.q[c] = qc;
    a.ga[c] = make_float4(gx[0] * iv, gy[0] * iv, gx[1] * iv, gy[1] * iv);
    a.gb[c] = make_float2(gx[2] * iv, gy[2] * iv);
}

// Viscous flux of flux face fi (interior or no-slip adiabatic wall; zero on
// other boundaries): mean gradient corrected along the centre line, Stokes
// stresses, Sutherland or constant viscosity, Fourier heat flux.
__device__ __forceinline__ void visc32_face(const Visc32Args& a, int fi, int2 lr, bool wall, const float n[2],
                                            float Fv[4]) {
    const float4 qL = a.q[lr.x];
    float4 qR;
    float gf[6];
    {
        const float4 l0 = a.ga[lr.x];
        const float2 l1 = a.gb[lr.x];
        if (lr.y >= 0) {
            qR = a.q[lr.y];
            const float4 r0 = a.ga[lr.y];
            const float2 r1 = a.gb[lr.y];
            gf[0] = 0.5f * (l0.x + r0.x);
            gf[1] = 0.5f * (l0.y + r0.y);
            gf[2] = 0.5f * (l0.z + r0.z);
            gf[3] = 0.5f * (l0.w + r0.w);
            gf[4] = 0.5f * (l1.x + r1.x);
            gf[5] = 0.5f * (l1.y + r1.y);
        } else {
            qR = make_float4(0.0f, 0.0f, qL.z, 0.0f);
            gf[0] = l0.x; gf[1] = l0.y; gf[2] = l0.z; gf[3] = l0.w; gf[4] = l1.x; gf[5] = l1.y;
        }
    }
    const float4 gg = a.fgeo[fi];
    const float idl = a.fgeo2[fi].y;
    const float dq[3] = {qR.x - qL.x, qR.y - qL.y, qR.z - qL.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float corr = dq[k] * idl - (gf[2 * k] * gg.z + gf[2 * k + 1] * gg.w);
        gf[2 * k] = fmaf(corr, gg.z, gf[2 * k]);
        gf[2 * k + 1] = fmaf(corr, gg.w, gf[2 * k + 1]);
    }
    const float u = 0.5f * (qL.x + qR.x), v = 0.5f * (qL.y + qR.y), T = 0.5f * (qL.z + qR.z);
    float mu = a.mu_ref;
    if (a.S > 0.0f) {
        const float r = T / a.T_ref;
        mu = a.mu_ref * (r * sqrtf(r)) * ((a.T_ref + a.S) / (T + a.S));
    }
    const float kc = mu * a.cp_over_pr;
    const float div = gf[0] + gf[3];
    const float txx = mu * (2.0f * gf[0] - (2.0f / 3.0f) * div);
    const float tyy = mu * (2.0f * gf[3] - (2.0f / 3.0f) * div);
    const float txy = mu * (gf[1] + gf[2]);
    Fv[0] = 0.0f;
    Fv[1] = txx * n[0] + txy * n[1];
    Fv[2] = txy * n[0] + tyy * n[1];
    Fv[3] = wall ? 0.0f : (u * txx + v * txy + kc * gf[4]) * n[0] + (u * txy + v * tyy + kc * gf[5]) * n[1];
}

// Flux of one face (local index fi) into G; VISC: minus the viscous flux.
// Positivity test of the face-state fallback in FP32 without divisions:
// density positive and 2 rho E > |rho u|^2 (pressure positive).
__device__ __forceinline__ bool admissible32(const float* W) {
    const float m2 = fmaf(W[1], W[1], W[2] * W[2]);
    return W[0] > 0.0f && 2.0f * W[0] * W[3] > m2;
}

// One quadrature point q of face fi: its flux Ft before the weight (the
// face states, the positivity fallback to the cell averages, the boundary
// condition's right state, the Riemann flux).
template <int RS, int NQ, class IX>
__device__ __forceinline__ void flux32_point(const FluxArgs& a, const float* __restrict__ fv, const GasParams& g,
                                             const BcTable& bct, int fi, int q, int2 lr, const float* n, int bi,
                                             int type, const IX& ix, const double* __restrict__ Ust, float* Ft) {
    const float gam = g.gamma_f;
    const float4* fq = reinterpret_cast<const float4*>(fv + (ix.f(fi) * NQ + q) * 8);
    float cl[4], cr[4], pl[5], pr[5];
    {
        const float4 x = fq[0];
        cl[0] = x.x; cl[1] = x.y; cl[2] = x.z; cl[3] = x.w;
    }
    if (type < 0) {
        const float4 x = fq[1];
        cr[0] = x.x; cr[1] = x.y; cr[2] = x.z; cr[3] = x.w;
    }
    if (!admissible32(cl))
#pragma unroll
        for (int i = 0; i < 4; i++) cl[i] = f(Ust[ix.u(lr.x) * NC + i]);
    if (type < 0 && !admissible32(cr))
#pragma unroll
        for (int i = 0; i < 4; i++) cr[i] = f(Ust[ix.u(lr.y) * NC + i]);
    primitives_guarded(g, cl, pl);
    if (type == MGPU_BC_WALL_ADIABATIC) {
        Ft[0] = 0.0f;
        Ft[1] = pl[2] * n[0];
        Ft[2] = pl[2] * n[1];
        Ft[3] = 0.0f;
        return;
    }
    if (type < 0) {
        primitives_guarded(g, cr, pr);
    } else if (type == MGPU_BC_SYMMETRY) {
#pragma unroll
        for (int i = 0; i < 4; i++) cr[i] = cl[i];
#pragma unroll
        for (int i = 0; i < NPR; i++) pr[i] = pl[i];
        const float un = pl[0] * n[0] + pl[1] * n[1];
        pr[0] = pl[0] - 2.0f * un * n[0];
        pr[1] = pl[1] - 2.0f * un * n[1];
    } else if (type == MGPU_BC_EXTRAPOLATION) {
#pragma unroll
        for (int i = 0; i < 4; i++) cr[i] = cl[i];
#pragma unroll
        for (int i = 0; i < NPR; i++) pr[i] = pl[i];
    } else if (type == MGPU_BC_UPT) {
        const double* d = bct.bc[bi].data;
        cr[0] = f(d[0]);
#pragma unroll
        for (int i = 0; i < NPR; i++) pr[i] = f(d[i + 1]);
    } else {  // MGPU_BC_P_OUT
        const float rho_l = cl[0];
        const float um = sqrtf(pl[0] * pl[0] + pl[1] * pl[1]);
        const float sos = sqrtf(gam * pl[2] / rho_l);
        const float po = (um < sos) ? f(bct.bc[bi].data[0]) : pl[2];
        const float T = pl[3];
        const float rho = po / (g.R_f * T);
        const float e = g.cv_f * T;
        cr[0] = rho;
        pr[0] = pl[0];
        pr[1] = pl[1];
        pr[2] = po;
        pr[3] = T;
        pr[4] = e + po / rho;
    }
    riemann<RS>(Ft, n, cl[0], pl, pl[2], gam, pl[4], cr[0], pr, pr[2], gam, pr[4], a.guard != 0);
}

// G of face fi from its weighted point sum F (times 1/2: the Gauss weights
// sum to 2) and, on viscous faces, the viscous flux.  half: 0 writes
// G[0..1], 1 writes G[2..3], 2 writes all four.  FP32 -> FP64 exactly on the
// integer pipe (f64_of), products in FP64.
__device__ __forceinline__ void store_G32(double* Gf4, double area, const float* F, const float* Fv, int half) {
    double2* Gf = reinterpret_cast<double2*>(Gf4);
    const double v1 = Fv ? area * f64_of(Fv[1]) : 0.0, v2 = Fv ? area * f64_of(Fv[2]) : 0.0,
                 v3 = Fv ? area * f64_of(Fv[3]) : 0.0;
    if (half != 1) {
        const double g1 = area * f64_of(F[1] * 0.5f);
        Gf[0] = make_double2(area * f64_of(F[0] * 0.5f), Fv ? g1 - v1 : g1);
    }
    if (half != 0) {
        const double g2 = area * f64_of(F[2] * 0.5f), g3 = area * f64_of(F[3] * 0.5f);
        Gf[1] = make_double2(Fv ? g2 - v2 : g2, Fv ? g3 - v3 : g3);
    }
}

template <int RS, int NQ, bool VISC, class IX>
__device__ __forceinline__ void flux32_face(const FluxArgs& a, const float* __restrict__ fv, const GasParams& g,
                                            const BcTable& bct, int fi, const IX& ix, const double* __restrict__ Ust,
                                            double* __restrict__ Gout, const Visc32Args* va = nullptr) {
    const int2 lr = a.lr[fi];
    const float2 nn = a.nrm32[fi];
    const float n[2] = {nn.x, nn.y};
    const int bi = a.bc[fi];
    const int type = bi < 0 ? -1 : bct.bc[bi].type;
    float F[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        float Ft[4];
        flux32_point<RS, NQ>(a, fv, g, bct, fi, q, lr, n, bi, type, ix, Ust, Ft);
#pragma unroll
        for (int i = 0; i < 4; i++) F[i] = fmaf(a.qw_f[q], Ft[i], F[i]);
    }
    const double area = a.area[fi];
    if (VISC && (type < 0 || type == MGPU_BC_WALL_ADIABATIC)) {
        float Fv[4];
        visc32_face(*va, fi, lr, type == MGPU_BC_WALL_ADIABATIC, n, Fv);
        store_G32(Gout + ix.f(fi) * 4, area, F, Fv, 2);
        return;
    }
    store_G32(Gout + ix.f(fi) * 4, area, F, nullptr, 2);
}

template <int RS, int NQ, bool VISC>
__global__ void __launch_bounds__(128) flux32_kernel(const FluxArgs a, const float* __restrict__ fv,
                                                     const GasParams g, const BcTable bct, const Visc32Args v) {
    const int fi = blockIdx.x * blockDim.x + threadIdx.x;
    if (fi >= a.n_faces) return;
    flux32_face<RS, NQ, VISC>(a, fv, g, bct, fi, Ix1{}, a.U, a.G, &v);
}

// Two lanes per face (two Gauss points): lane q computes point q's flux, the
// pair swaps them and both sum in the one-lane kernel's order (point 0
// first), so G is bit for bit flux32_kernel's; lane 0 stores the first half
// of the face's G, lane 1 the second.  Half the dependent work per thread,
// twice the faces in flight.
template <int RS, bool VISC>
__global__ void __launch_bounds__(128) flux32_pair_kernel(const FluxArgs a, const float* __restrict__ fv,
                                                          const GasParams g, const BcTable bct, const Visc32Args v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int fi = t >> 1, q = t & 1;
    const unsigned live = __ballot_sync(0xffffffffu, fi < a.n_faces);
    if (fi >= a.n_faces) return;
    const int2 lr = a.lr[fi];
    const float2 nn = a.nrm32[fi];
    const float n[2] = {nn.x, nn.y};
    const int bi = a.bc[fi];
    const int type = bi < 0 ? -1 : bct.bc[bi].type;
    float Ft[4], F[4];
    flux32_point<RS, 2>(a, fv, g, bct, fi, q, lr, n, bi, type, Ix1{}, a.U, Ft);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float o = __shfl_xor_sync(live, Ft[i], 1);
        const float f0 = q == 0 ? Ft[i] : o, f1 = q == 0 ? o : Ft[i];
        F[i] = fmaf(a.qw_f[1], f1, fmaf(a.qw_f[0], f0, 0.0f));
    }
    const double area = a.area[fi];
    if (VISC && (type < 0 || type == MGPU_BC_WALL_ADIABATIC)) {
        float Fv[4];
        visc32_face(v, fi, lr, type == MGPU_BC_WALL_ADIABATIC, n, Fv);
        store_G32(a.G + (size_t)fi * 4, area, F, Fv, q);
        return;
    }
    store_G32(a.G + (size_t)fi * 4, area, F, nullptr, q);
}

template <int RS, int NQ>
cudaError_t flux_go(const FluxArgs& a, const float* fv, const GasParams& g, const BcTable& bct,
                    const Visc32Args* v, cudaStream_t s) {
    const unsigned blocks = (unsigned)((a.n_faces + 127) / 128);
    if (!blocks) return cudaSuccess;
    if constexpr (NQ == 2) {
        const unsigned pblocks = (unsigned)((2ll * a.n_faces + 127) / 128);
        if (v) flux32_pair_kernel<RS, true><<<pblocks, 128, 0, s>>>(a, fv, g, bct, *v);
        else flux32_pair_kernel<RS, false><<<pblocks, 128, 0, s>>>(a, fv, g, bct, Visc32Args{});
        return cudaGetLastError();
    }
    if (v) flux32_kernel<RS, NQ, true><<<blocks, 128, 0, s>>>(a, fv, g, bct, *v);
    else flux32_kernel<RS, NQ, false><<<blocks, 128, 0, s>>>(a, fv, g, bct, Visc32Args{});
    return cudaGetLastError();
}

template <int RS>
cudaError_t flux_nq(const FluxArgs& a, const float* fv, const GasParams& g, const BcTable& bct, int nq,
                    const Visc32Args* v, cudaStream_t s) {
    switch (nq) {
        case 1: return flux_go<RS, 1>(a, fv, g, bct, v, s);
        case 2: return flux_go<RS, 2>(a, fv, g, bct, v, s);
    }
    return cudaErrorInvalidValue;
}

template <int K, int M, int NQ, bool SEL, int BS, int MINB, bool VG>
cudaError_t teno_go1(const TenoArgs& a, const float* U, float* fv, uint8_t* masks, const uint8_t* pred,
                     cudaStream_t s) {
    const long long threads = (long long)a.n_cells * 4;
    const unsigned blocks = (unsigned)((threads + BS - 1) / BS);
    if (blocks) teno32_kernel<K, M, NQ, SEL, BS, MINB, VG><<<blocks, BS, 0, s>>>(a, U, fv, masks, pred);
    return cudaGetLastError();
}

// Staged form (teno32_staged_kernel): one warp per tile, WARPS per block.
template <int K, int M, int NQ, bool SEL, int NSLOT, int WARPS, int MINB, bool VG>
cudaError_t teno_staged1(const TenoArgs& a, const float* U, float* fv, uint8_t* masks, const uint8_t* pred,
                         cudaStream_t s) {
    constexpr unsigned smem = WARPS * StageLayout<K, M, NQ, NSLOT>::WARP;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(teno32_staged_kernel<K, M, NQ, SEL, NSLOT, WARPS, MINB, VG>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long tiles = ((long long)a.n_cells + 7) / 8;
    const unsigned blocks = (unsigned)((tiles + WARPS - 1) / WARPS);
    if (blocks)
        teno32_staged_kernel<K, M, NQ, SEL, NSLOT, WARPS, MINB, VG><<<blocks, WARPS * 32, smem, s>>>(a, U, fv, masks, pred,
                                                                                               a.err);
    return cudaGetLastError();
}

// Launch shapes the autotuner chooses from: (block size, minimum resident
// blocks per SM), i.e. register caps of 128, 80 and 64 per thread; shapes
// 4-7 are the staged form (p = 3): one stencil slot per warp, 4 warps per
// block, at most 80 registers; two slots, 2 warps, 128; one slot, 4 warps,
// 128; one slot, 4 warps, at most 72 registers (7 blocks per SM).
template <int K, int M, int NQ, bool SEL, bool VG>
cudaError_t teno_go(const TenoArgs& a, const float* U, float* fv, uint8_t* masks, const uint8_t* pred, int shape,
                    cudaStream_t s) {
    switch (shape) {
        case 0: return teno_go1<K, M, NQ, SEL, 128, 4, VG>(a, U, fv, masks, pred, s);
        case 1: return teno_go1<K, M, NQ, SEL, 128, 6, VG>(a, U, fv, masks, pred, s);
        case 2: return teno_go1<K, M, NQ, SEL, 128, 8, VG>(a, U, fv, masks, pred, s);
        case 3: return teno_go1<K, M, NQ, SEL, 256, 4, VG>(a, U, fv, masks, pred, s);
    }
    if constexpr (K == 10 && M == 20 && NQ == 2) {
        if (shape == 4) return teno_staged1<K, M, NQ, SEL, 1, 4, 6, VG>(a, U, fv, masks, pred, s);
        if (shape == 5) return teno_staged1<K, M, NQ, SEL, 1, 2, 14, VG>(a, U, fv, masks, pred, s);
        if (shape == 6) return teno_staged1<K, M, NQ, SEL, 1, 1, 28, VG>(a, U, fv, masks, pred, s);
        if (shape == 7) return teno_staged1<K, M, NQ, SEL, 1, 4, 7, VG>(a, U, fv, masks, pred, s);
    }
    return cudaErrorInvalidValue;
}

// group of a batch thread index
__device__ __forceinline__ int batch_group(const long long* start, int n, long long gt) {
    int g = 0;
    while (g + 1 < n && gt >= start[g + 1]) ++g;
    return g;
}

// Batched reconstruction: thread (case, cell, variable), 32 consecutive
// threads = one 8-cell tile of one case, consecutive tiles = the same mesh
// tile of consecutive cases (so a table tile is reused from cache).
template <int K, int M, int NQ, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) teno32_batch_kernel(const BatchLaunch b, const float* __restrict__ U) {
    const long long total = b.teno0[b.n_groups];
    for (long long gt = (long long)blockIdx.x * BS + threadIdx.x; gt < total; gt += (long long)gridDim.x * BS) {
        const int gi = batch_group(b.teno0, b.n_groups, gt);
        const unsigned t = (unsigned)(gt - b.teno0[gi]);
        const int v = (int)(t & 3), lane8 = (int)((t >> 2) & 7);
        const unsigned tc = t >> 5, C = b.C[gi], cs = tc % C;
        const int cell = (int)(tc / C) * 8 + lane8;
        // frozen (failed) cases and cells past the mesh do no work; a warp is one case's tile
        const bool on = cell < b.n_cells[gi] && b.flags[b.case0[gi] + cs] == 0u;
        const unsigned live = __ballot_sync(0xffffffffu, on);
        if (!on) continue;
        GlobalSrc<K, M, NQ> src{b.teno[gi], cell >> 3};
        teno32_cell<K, M, NQ, false, false>(b.teno[gi], U, b.fv, nullptr, nullptr, cell, v, live,
                                     IxB{b.ubase[gi], b.fbase[gi], C, cs}, src);
    }
}

// Batched face flux, two lanes per (case, face) item (flux32_pair_kernel's
// scheme): the grid-stride loop runs whole warps, so every lane of a warp
// takes part in the pair exchange of each pass.
template <int RS>
__global__ void __launch_bounds__(128) flux32_pair_batch_kernel(const BatchLaunch b, const GasParams g,
                                                               const BcTable bct, const double* __restrict__ U) {
    const long long total = 2 * b.face0[b.n_groups];
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * 128 + (threadIdx.x & ~31); base < total;
         base += (long long)gridDim.x * 128) {
        const long long gt = base + lane;
        bool on = gt < total;
        int gi = 0, fi = 0;
        unsigned C = 1, cs = 0;
        if (on) {
            const long long item = gt >> 1;
            gi = batch_group(b.face0, b.n_groups, item);
            const unsigned t = (unsigned)(item - b.face0[gi]);
            const unsigned tc = t >> 3;
            C = b.C[gi];
            cs = tc % C;
            fi = (int)(tc / C) * 8 + (int)(t & 7);
            on = fi < b.n_faces[gi] && b.flags[b.case0[gi] + cs] == 0u;
        }
        const unsigned live = __ballot_sync(0xffffffffu, on);
        if (!on) continue;
        const int q = (int)(gt & 1);
        const FluxArgs& a = b.flux[gi];
        const IxB ix{b.ubase[gi], b.fbase[gi], C, cs};
        const int2 lr = a.lr[fi];
        const float2 nn = a.nrm32[fi];
        const float n[2] = {nn.x, nn.y};
        const int bi = a.bc[fi];
        const int type = bi < 0 ? -1 : bct.bc[bi].type;
        float Ft[4], F[4];
        flux32_point<RS, 2>(a, b.fv, g, bct, fi, q, lr, n, bi, type, ix, U, Ft);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const float o = __shfl_xor_sync(live, Ft[i], 1);
            const float f0 = q == 0 ? Ft[i] : o, f1 = q == 0 ? o : Ft[i];
            F[i] = fmaf(a.qw_f[1], f1, fmaf(a.qw_f[0], f0, 0.0f));
        }
        store_G32(b.G + ix.f(fi) * 4, a.area[fi], F, nullptr, q);
    }
}

// Batched reconstruction, staged (teno32_staged_kernel's scheme): one warp
// per (group, mesh tile, case); the C cases of a mesh tile are consecutive
// warps, so their bulk copies of the tile's table blocks come from L2 after
// the first.  A case that is frozen skips the warp; a wait that runs out
// sets bit 2 of the case's flags (which then freezes it).
template <int K, int M, int NQ, int NSLOT, int WARPS, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) teno32_batch_staged_kernel(const BatchLaunch b,
                                                                               const float* __restrict__ U) {
    using L = StageLayout<K, M, NQ, NSLOT>;
    using B = TileBlocks<K, M, NQ>;
    extern __shared__ __align__(128) uint8_t stage_smem[];
    const int w = threadIdx.x >> 5, lane32 = threadIdx.x & 31;
    const long long gt = ((long long)blockIdx.x * WARPS + w) * 32;  // the warp's first item
    if (gt >= b.teno0[b.n_groups]) return;
    const int gi = batch_group(b.teno0, b.n_groups, gt);
    const unsigned tc = (unsigned)(gt - b.teno0[gi]) >> 5, C = b.C[gi], cs = tc % C;
    const int tile = (int)(tc / C);
    const unsigned gc = b.case0[gi] + cs;
    if (b.flags[gc] != 0u) return;
    const TenoArgs& a = b.teno[gi];
    StageSrc<K, M, NQ, NSLOT> src{a, stage_smem + (size_t)w * L::WARP, tile, lane32};
    if (lane32 == 0) {
        for (int i = 0; i <= NSLOT; ++i) mbar_init(src.bar(i), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbar_expect_tx(src.bar(NSLOT), B::CB);
        bulk_g2s(src.base + L::PHI, reinterpret_cast<const char*>(a.fcode) + (size_t)tile * B::CB, B::CB, src.bar(NSLOT));
    }
    __syncwarp();
    src.prefetch_central();
    const int cell = tile * 8 + (lane32 >> 2), v = lane32 & 3;
    teno32_cell<K, M, NQ, false, false>(a, U, b.fv, nullptr, nullptr, cell, v, 0xffffffffu,
                                 IxB{b.ubase[gi], b.fbase[gi], C, cs}, src, cell < b.n_cells[gi]);
    if (!src.ok) {
        if (lane32 == 0) atomicOr(b.flags + gc, 4u);
        for (int i = 0; i <= NSLOT; ++i) {
            const int uses = i == NSLOT ? 1 : (i < src.issued ? (src.issued - i + NSLOT - 1) / NSLOT : 0);
            if (uses > 0) mbar_wait(src.bar(i), (unsigned)(uses - 1) & 1u);
        }
    }
}

// Table source of teno32_cell: every stencil block of the tile resident in
// the CTA's shared memory (slot s = stencil s), loaded once.
template <int K, int M, int NQ>
struct ResidentSrc {
    using B = TileBlocks<K, M, NQ>;
    using L = StageLayout<K, M, NQ, 4>;
    const uint8_t* base;
    unsigned need_all;
    __device__ __forceinline__ unsigned tile_need(unsigned) const { return need_all; }
    __device__ __forceinline__ bool begin(int) { return true; }
    __device__ __forceinline__ void end(int) {}
    __device__ __forceinline__ const uint4* nb(int s) const {
        return reinterpret_cast<const uint4*>(base + s * L::SLOT + B::PB);
    }
    __device__ __forceinline__ const float4* P(int s) const { return reinterpret_cast<const float4*>(base + s * L::SLOT); }
    __device__ __forceinline__ const uint16_t* codes() { return reinterpret_cast<const uint16_t*>(base + L::PHI); }
    template <class T>
    __device__ __forceinline__ T ld(const T* p) const { return *p; }
};

// Batched reconstruction with resident tables: one CTA per (mesh group,
// mesh tile).  The tile's table blocks are bulk-copied into shared memory
// once; the CTA's warps then take the group's cases in turn (case w, w +
// WARPS, ...), so a table byte crosses from L2 once per tile instead of
// once per case.  Frozen cases are skipped; a wait that runs out flags the
// group's cases (bit 2).
template <int K, int M, int NQ, int WARPS, int MINB>
__global__ void __launch_bounds__(WARPS * 32, MINB) teno32_batch_resident_kernel(const BatchLaunch b,
                                                                                 const float* __restrict__ U) {
    using L = StageLayout<K, M, NQ, 4>;
    using B = TileBlocks<K, M, NQ>;
    extern __shared__ __align__(128) uint8_t stage_smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(stage_smem + L::BAR);
    long long t = blockIdx.x;
    int gi = 0;
    while (gi + 1 < b.n_groups && t >= (long long)((b.n_cells[gi] + 7) / 8)) {
        t -= (b.n_cells[gi] + 7) / 8;
        ++gi;
    }
    const int tile = (int)t, n = b.n_cells[gi];
    const TenoArgs& a = b.teno[gi];
    unsigned need_all = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (tile * 8 + k < n) need_all |= a.smask[tile * 8 + k];
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        unsigned bytes = B::CB;
        for (int s = 0; s < B::S; ++s)
            if ((need_all >> s) & 1u) bytes += L::SLOT;
        mbar_expect_tx(bar, bytes);
        bulk_g2s(stage_smem + L::PHI, reinterpret_cast<const char*>(a.fcode) + (size_t)tile * B::CB, B::CB, bar);
        for (int s = 0; s < B::S; ++s) {
            if (!((need_all >> s) & 1u)) continue;
            bulk_g2s(stage_smem + s * L::SLOT, reinterpret_cast<const char*>(a.P4) + (size_t)(tile * B::S + s) * B::PB,
                     B::PB, bar);
            bulk_g2s(stage_smem + s * L::SLOT + B::PB,
                     reinterpret_cast<const char*>(a.nb4) + (size_t)(tile * B::S + s) * B::NBB, B::NBB, bar);
        }
    }
    __syncthreads();
    const bool ok = __syncthreads_and(mbar_wait(bar, 0));
    const unsigned C = b.C[gi];
    if (!ok) {
        if (threadIdx.x == 0)
            for (unsigned cs = 0; cs < C; ++cs) atomicOr(b.flags + b.case0[gi] + cs, 4u);
        mbar_wait(bar, 0);
        return;
    }
    ResidentSrc<K, M, NQ> src{stage_smem, need_all};
    const int warp = threadIdx.x >> 5, lane32 = threadIdx.x & 31;
    const int cell = tile * 8 + (lane32 >> 2), v = lane32 & 3;
    for (unsigned cs = warp; cs < C; cs += WARPS) {
        if (b.flags[b.case0[gi] + cs] != 0u) continue;
        teno32_cell<K, M, NQ, false, false>(a, U, b.fv, nullptr, nullptr, cell, v, 0xffffffffu,
                                     IxB{b.ubase[gi], b.fbase[gi], C, cs}, src, cell < n);
    }
}

template <int K, int M, int NQ, int WARPS, int MINB>
cudaError_t teno_batch_resident(const BatchLaunch& b, const float* U, cudaStream_t s) {
    constexpr unsigned smem = StageLayout<K, M, NQ, 4>::WARP;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(teno32_batch_resident_kernel<K, M, NQ, WARPS, MINB>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    long long tiles = 0;
    for (int g = 0; g < b.n_groups; ++g) tiles += (b.n_cells[g] + 7) / 8;
    if (tiles > 0)
        teno32_batch_resident_kernel<K, M, NQ, WARPS, MINB><<<(unsigned)tiles, WARPS * 32, smem, s>>>(b, U);
    return cudaGetLastError();
}

template <int K, int M, int NQ, int NSLOT, int WARPS, int MINB>
cudaError_t teno_batch_staged(const BatchLaunch& b, const float* U, cudaStream_t s) {
    constexpr unsigned smem = WARPS * StageLayout<K, M, NQ, NSLOT>::WARP;
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(teno32_batch_staged_kernel<K, M, NQ, NSLOT, WARPS, MINB>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long warps = b.teno0[b.n_groups] / 32;
    const long long blocks = (warps + WARPS - 1) / WARPS;
    if (blocks > 0) teno32_batch_staged_kernel<K, M, NQ, NSLOT, WARPS, MINB><<<(unsigned)blocks, WARPS * 32, smem, s>>>(b, U);
    return cudaGetLastError();
}

template <int K, int M, int NQ, int BS, int MINB>
cudaError_t teno_batch_go(const BatchLaunch& b, const float* U, int blocks_per_sm, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (b.teno0[b.n_groups] + BS - 1) / BS;
    long long blocks = blocks_per_sm > 0 ? (long long)sms * blocks_per_sm : need;
    if (blocks > need) blocks = need;
    if (blocks > 0) teno32_batch_kernel<K, M, NQ, BS, MINB><<<(unsigned)blocks, BS, 0, s>>>(b, U);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_teno_batch(const BatchLaunch& b, const float* U, int shape, int blocks_per_sm, cudaStream_t s) {
    switch (shape) {
        case 0: return teno_batch_go<10, 20, 2, 128, 4>(b, U, blocks_per_sm, s);
        case 1: return teno_batch_go<10, 20, 2, 128, 6>(b, U, blocks_per_sm, s);
        case 2: return teno_batch_go<10, 20, 2, 128, 8>(b, U, blocks_per_sm, s);
        case 3: return teno_batch_go<10, 20, 2, 256, 4>(b, U, blocks_per_sm, s);
        case 4: return teno_batch_staged<10, 20, 2, 1, 4, 6>(b, U, s);
        case 5: return teno_batch_staged<10, 20, 2, 2, 2, 7>(b, U, s);
        case 6: return teno_batch_staged<10, 20, 2, 1, 4, 4>(b, U, s);
        case 7: return teno_batch_resident<10, 20, 2, 4, 6>(b, U, s);
        case 8: return teno_batch_resident<10, 20, 2, 8, 3>(b, U, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_flux_batch(const BatchLaunch& b, const GasParams& g, const BcTable& bct, int rsolver, int nq,
                              const double* U, cudaStream_t s) {
    if (nq != 2) return cudaErrorInvalidValue;
    const long long blocks = (2 * b.face0[b.n_groups] + 127) / 128;
    if (blocks == 0) return cudaSuccess;
    switch (rsolver) {
        case MGPU_RIEMANN_RUSANOV:
            flux32_pair_batch_kernel<MGPU_RIEMANN_RUSANOV><<<(unsigned)blocks, 128, 0, s>>>(b, g, bct, U);
            break;
        case MGPU_RIEMANN_HLL: flux32_pair_batch_kernel<MGPU_RIEMANN_HLL><<<(unsigned)blocks, 128, 0, s>>>(b, g, bct, U); break;
        case MGPU_RIEMANN_HLLC:
            flux32_pair_batch_kernel<MGPU_RIEMANN_HLLC><<<(unsigned)blocks, 128, 0, s>>>(b, g, bct, U);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_teno(const TenoArgs& a, int K, int M, int nq, const float* U, float* fv, uint8_t* masks,
                        int shape, cudaStream_t s) {
    // viscous gradients from the reconstruction in their own instantiations
    if (a.vq) {
        if (K == 10 && M == 20 && nq == 2) return teno_go<10, 20, 2, false, true>(a, U, fv, masks, nullptr, shape, s);
        if (K == 6 && M == 12 && nq == 1) return teno_go1<6, 12, 1, false, 128, 4, true>(a, U, fv, masks, nullptr, s);
        if (K == 3 && M == 6 && nq == 1) return teno_go1<3, 6, 1, false, 128, 4, true>(a, U, fv, masks, nullptr, s);
        return cudaErrorInvalidValue;
    }
    if (K == 10 && M == 20 && nq == 2) return teno_go<10, 20, 2, false, false>(a, U, fv, masks, nullptr, shape, s);
    if (K == 6 && M == 12 && nq == 1) return teno_go1<6, 12, 1, false, 128, 4, false>(a, U, fv, masks, nullptr, s);
    if (K == 3 && M == 6 && nq == 1) return teno_go1<3, 6, 1, false, 128, 4, false>(a, U, fv, masks, nullptr, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_teno_selected(const TenoArgs& a, int K, int M, int nq, const float* U, const uint8_t* pred,
                                 float* fv, uint8_t* masks, int shape, cudaStream_t s) {
    if (K == 10 && M == 20 && nq == 2)
        return a.vq ? teno_go<10, 20, 2, true, true>(a, U, fv, masks, pred, shape, s)
                    : teno_go<10, 20, 2, true, false>(a, U, fv, masks, pred, shape, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_flux(const FluxArgs& a, const float* fv, const GasParams& g, const BcTable& bct, int rsolver,
                        int nq, const Visc32Args* visc, cudaStream_t s) {
    switch (rsolver) {
        case MGPU_RIEMANN_RUSANOV: return flux_nq<MGPU_RIEMANN_RUSANOV>(a, fv, g, bct, nq, visc, s);
        case MGPU_RIEMANN_HLL: return flux_nq<MGPU_RIEMANN_HLL>(a, fv, g, bct, nq, visc, s);
        case MGPU_RIEMANN_HLLC: return flux_nq<MGPU_RIEMANN_HLLC>(a, fv, g, bct, nq, visc, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_visc_grad(const Visc32Args& v, const BcTable& bct, const float* U, cudaStream_t s) {
    if (v.n_cells > 0) visc_grad32_kernel<<<(v.n_cells + 255) / 256, 256, 0, s>>>(v, bct, U);
    return cudaGetLastError();
}

}  // namespace f32
}  // namespace mgpu
