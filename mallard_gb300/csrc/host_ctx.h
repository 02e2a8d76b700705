// host_ctx.h -- the solver context (struct mgpu_ctx) and the host helpers
// shared by the translation units behind the C ABI.
#pragma once

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.h"
#include "host.h"
#include "selector_launch.h"

namespace mgpu {

struct CudaFail : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct ArgFail : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct Unsupported : std::runtime_error {
    using std::runtime_error::runtime_error;
};

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaFail(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        ck(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
        n = count;
        ck(cudaMemset(p, 0, count * sizeof(T)), "cudaMemset");
    }
    void upload(const std::vector<T>& v) {
        alloc(v.size());
        if (!v.empty()) ck(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    }
    size_t bytes() const { return n * sizeof(T); }
};

struct BcHost {
    uint32_t zone;
    int type;
    double data[6];
};


}  // namespace mgpu

using namespace mgpu;

struct mgpu_ctx {
    mgpu_config cfg{};
    HostMesh mesh;
    std::vector<BcHost> bcs;
    bool finalized = false;
    GasParams gas{};
    BcTable bct{};
    int nq = 1, K = 0, M = 0;
    double qw[4] = {0, 0, 0, 0};

    cudaStream_t stream = nullptr;
    bool own_stream = false;

    // numbering: internal <-> caller
    uint32_t N = 0;
    std::vector<uint32_t> cell_new, cell_old;
    uint32_t F_flux = 0, F_real = 0;
    std::vector<int32_t> face_new;
    std::vector<uint32_t> face_old;

    // device state and work arrays
    DevArray<double> U, Ut, W, prim, vol, fv, G, rho_cell, rhs, scal;  // scal: dt, t
    DevArray<float> fv32;        // face states of the FP32-bulk form
    DevArray<float> U32, Ut32;   // FP32 copies of U and Ut (FP32-bulk form)
    // learned stencil selector (FP32 form): weight image, predictions
    bool sel_on = false;
    float sel_thr_central = 0.0f, sel_thr_directional = 0.0f;
    bool sel_every_stage = false;
    uint32_t sel_interval = 1;  // steps per selector prediction
    int teno_shape = 0;  // FP32 reconstruction launch shape (mgpu_autotune)
    DevArray<uint8_t> sel_wimg, pred, trusted;  // raw predictions, after the neighbour check
    DevArray<unsigned> sel_err;
    DevArray<unsigned> flags;
    DevArray<unsigned long long> rmax;
    DevArray<int2> lr;
    DevArray<double2> nrm;
    DevArray<float2> nrm32;  // FP32 form: the unit normals rounded once
    DevArray<float4> geo32;  // FP32 form: unit normal and 1 / dxn rounded once (time step)
    DevArray<double> area, dxn, idxn, ivol, snd;
    // viscous flux: cell centres, face midpoints, gradients
    DevArray<double2> xc, xf;
    DevArray<double> grad;
    ViscArgs visc{};
    // FP32 form: face geometry and per-cell (u, v, T) and gradients
    DevArray<float4> vgeo, vq, vga;
    DevArray<float2> vgeo2, vgb;
    Visc32Args visc32{};
    // viscous gradients from the reconstruction: per cell the inverse
    // Jacobian of its reference frame
    DevArray<double> ji;
    DevArray<float4> ji4;
    DevArray<int8_t> bcidx;
    DevArray<int4> gat, cfaces;
    DevArray<uint32_t> nb, cface;
    DevArray<double> ar, P, phi;
    DevArray<uint32_t> nb4;
    DevArray<float> P4;
    DevArray<uint16_t> fcode;   // FP32 form: face-shape code per cell (3 bits per face slot)
    DevArray<float4> phi_tab4;  // FP32 form: the 8 code slots' shape sets
    DevArray<uint8_t> smask, masks, bcell;
    DevArray<double> staging;      // caller-order rows for state transfers
    DevArray<uint32_t> perm_old;   // internal cell -> caller cell
    DevArray<uint32_t> perm_new;   // caller cell -> internal cell
    TenoArgs teno{};

    // CUDA graphs of one CFL step, keyed by cfl: with the selector's
    // prediction, and (prediction interval > 1) without it
    cudaGraphExec_t step_exec = nullptr, step_exec_np = nullptr;
    double step_cfl = -1.0;
    void drop_graphs() {
        if (step_exec) cudaGraphExecDestroy(step_exec);
        if (step_exec_np) cudaGraphExecDestroy(step_exec_np);
        step_exec = step_exec_np = nullptr;
    }

    // per-launch timing
    bool timing = false;
    struct Mark {
        int cls;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;
    size_t marks_used = 0;
    double recon_bytes = 0, stage_bytes = 0;

    ~mgpu_ctx() {
        drop_graphs();
        for (auto& m : marks) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        if (own_stream && stream) cudaStreamDestroy(stream);
    }

    double* dt_ptr() { return scal.p; }
    double* t_ptr() { return scal.p + 1; }

    // ---- launch helpers ---------------------------------------------------
    template <class F>
    void timed(int cls, F&& launch) {
        if (!timing) {
            ck(launch(), "kernel launch");
            return;
        }
        if (marks_used == marks.size()) {
            Mark m{cls, nullptr, nullptr};
            ck(cudaEventCreate(&m.a), "cudaEventCreate");
            ck(cudaEventCreate(&m.b), "cudaEventCreate");
            marks.push_back(m);
        }
        Mark& m = marks[marks_used++];
        m.cls = cls;
        ck(cudaEventRecord(m.a, stream), "cudaEventRecord");
        ck(launch(), "kernel launch");
        ck(cudaEventRecord(m.b, stream), "cudaEventRecord");
    }

    bool fast() const { return cfg.precision == MGPU_PREC_FP64_FAST; }
    // the viscous flux's cell gradients come from the reconstruction
    bool recon_grads() const {
        return cfg.viscous && cfg.recon == MGPU_RECON_TENO && cfg.viscous_gradients == MGPU_VISC_GRAD_RECON;
    }
    bool single() const { return cfg.precision == MGPU_PREC_FP32; }
    // reciprocal-based update and time step (every form but the exact one)
    bool rcp() const { return cfg.precision != MGPU_PREC_FP64; }

    // predict: run the selector on Uin (otherwise reuse its last predictions)
    void reconstruct(const double* Uin, uint8_t* mask_out, bool predict = true) {
        const float* u32 = Uin == U.p ? U32.p : Ut32.p;  // the FP32 form reads the FP32 copy
        if (single() && sel_on) {
            if (predict) {
                timed(4, [&] {
                    return sel::launch_mlp_cells(sel_wimg.p, teno, u32, sel_thr_central, sel_thr_directional, pred.p,
                                                 sel_err.p, stream);
                });
                timed(4, [&] { return sel::launch_trust((int)N, cfaces.p, lr.p, pred.p, trusted.p, stream); });
            }
            timed(0, [&] {
                return f32::launch_teno_selected(teno, K, M, nq, u32, trusted.p, fv32.p, mask_out, teno_shape,
                                                 stream);
            });
        } else if (single()) {
            timed(0, [&] { return f32::launch_teno(teno, K, M, nq, u32, fv32.p, mask_out, teno_shape, stream); });
        } else if (cfg.recon == MGPU_RECON_TENO) {
            timed(0, [&] {
                return fast() ? fast::launch_teno(teno, K, M, nq, cfg.teno_variant, Uin, fv.p, mask_out, stream)
                              : exact::launch_teno(teno, K, M, nq, cfg.teno_variant, Uin, fv.p, mask_out, stream);
            });
        } else {
            timed(0, [&] { return launch_first_order((int)F_flux, lr.p, Uin, fv.p, stream); });
        }
    }

    // viscous face flux into G (after the inviscid flux of the same stage);
    // the FP32 form computes the gradients before the flux, whose kernel
    // subtracts the viscous flux itself
    void viscous(const double* Uin) {
        if (!cfg.viscous || single()) return;
        timed(1, [&] { return launch_visc(Uin); });
    }
    void viscous_gradients32(const float* Uin) {
        if (!cfg.viscous || recon_grads()) return;
        timed(1, [&] { return f32::launch_visc_grad(visc32, bct, Uin, stream); });
    }
    cudaError_t launch_visc(const double* Uin) { return launch_viscous(visc, gas, bct, Uin, stream); }

    void flux(const double* Uin) {
        FluxArgs a{};
        a.n_faces = (int)F_flux;
        a.lr = lr.p;
        a.nrm = nrm.p;
        a.nrm32 = nrm32.p;
        a.area = area.p;
        a.bc = bcidx.p;
        a.fv = fv.p;
        a.G = G.p;
        a.U = Uin;
        for (int i = 0; i < 4; i++) {
            a.qw[i] = qw[i];
            a.qw_f[i] = (float)qw[i];
        }
        const bool pos = cfg.recon == MGPU_RECON_TENO && cfg.teno_variant != MGPU_TENO_REFERENCE;
        a.guard = cfg.recon == MGPU_RECON_TENO && cfg.teno_variant == MGPU_TENO_ROBUST;
        if (single()) {
            viscous_gradients32(Uin == U.p ? U32.p : Ut32.p);
            const Visc32Args* v = cfg.viscous ? &visc32 : nullptr;
            timed(1, [&] { return f32::launch_flux(a, fv32.p, gas, bct, cfg.riemann_solver, nq, v, stream); });
            return;
        }
        timed(1, [&] {
            return fast() ? fast::launch_flux(a, gas, bct, cfg.riemann_solver, nq, pos, stream)
                          : exact::launch_flux(a, gas, bct, cfg.riemann_solver, nq, pos, stream);
        });
    }

    UpdateArgs update_args() {
        UpdateArgs a{};
        a.n_cells = (int)N;
        a.gat = gat.p;
        a.G = G.p;
        a.vol = vol.p;
        a.ivol = ivol.p;
        a.dt = dt_ptr();
        a.U = U.p;
        a.Ut = Ut.p;
        a.W = W.p;
        // the FP32 form writes no FP64 primitives in its steps (refresh_prims)
        a.prim = single() ? nullptr : prim.p;
        a.snd = single() ? nullptr : snd.p;
        a.rhs = rhs.p;
        a.flags = flags.p;
        return a;
    }

    // stages of one step: FE 1, SSPRK3 3, RK4 4
    int n_stages() const {
        return cfg.time_integrator == MGPU_INTEGRATOR_FE ? 1 : (cfg.time_integrator == MGPU_INTEGRATOR_RK4 ? 4 : 3);
    }

    void stage(int k, bool predict_step = true) {
        const double* in = (k == 1) ? U.p : Ut.p;
        // the selector predicts at the first stage of a prediction step (every
        // sel_interval-th), from the step's initial state, or at every stage
        // when asked to
        reconstruct(in, nullptr, (k == 1 && predict_step) || sel_every_stage);
        flux(in);
        viscous(in);
        UpdateArgs a = update_args();
        if (single()) a.u32 = k == n_stages() ? U32.p : Ut32.p;
        timed(2, [&] { return launch_update(a, gas, k, cfg.time_integrator, rcp(), stream); });
    }

    void spectral_and_dt(double cfl, bool accumulate_t) {
        ck(cudaMemsetAsync(rmax.p, 0, sizeof(unsigned long long), stream), "cudaMemsetAsync");
        SpecArgs s{};
        s.n_cells = (int)N;
        s.cfaces = cfaces.p;
        s.lr = lr.p;
        s.nrm = nrm.p;
        s.dxn = dxn.p;
        s.idxn = idxn.p;
        s.U = U.p;
        s.prim = prim.p;
        s.snd = snd.p;
        s.rho_cell = rho_cell.p;
        s.rmax_bits = rmax.p;
        spec_fp32(s);
        timed(3, [&] { return launch_spectral(s, rcp(), stream); });
        ck(launch_dt(rmax.p, cfl, dt_ptr(), accumulate_t ? t_ptr() : nullptr, flags.p, stream), "dt launch");
    }

    // Gas constants of the spectral radius; in the FP32 form, its FP32 state
    // rows (the radius is then computed from them in FP32).
    void spec_fp32(SpecArgs& s) const {
        s.gamma = gas.gamma;
        s.p_min = gas.p_min;
        s.p_max = gas.p_max;
        s.gamma_f = gas.gamma_f;
        s.p_min_f = gas.p_min_f;
        s.p_max_f = gas.p_max_f;
        s.idxn = idxn.p;
        s.u32 = single() ? reinterpret_cast<const float4*>(U32.p) : nullptr;
        s.geo32 = single() ? geo32.p : nullptr;
    }

    // The FP32 form's steps leave the FP64 primitives and sound speeds
    // behind (nothing in its step reads them); they are recovered from U,
    // with the reference's formula, when a caller asks for them.
    bool prim_stale = false;
    void refresh_prims() {
        if (!prim_stale) return;
        ck(launch_primitives_batch(gas, N, U.p, prim.p, stream), "primitives");
        ck(launch_sound((int)N, gas.gamma, U.p, prim.p, snd.p, stream), "sound speed");
        prim_stale = false;
    }

    void cfl_step(double cfl, bool predict_step = true) {
        spectral_and_dt(cfl, true);
        for (int k = 1; k <= n_stages(); ++k) stage(k, predict_step);
    }

    // ---- host <-> device in caller numbering ------------------------------
    // Pinned host memory: one kernel pass reads (or writes) the caller's
    // rows in place and permutes them.  Other memory: one copy-engine
    // transfer into a staging array, then a permutation kernel.  Uploads are
    // not synchronised: stream order protects the staging array, and every
    // caller synchronises before it returns (the host buffer is borrowed
    // until then).
    // The device's address of pinned host memory (null for other memory).
    static const double* pinned_view(const double* h) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return at.type == cudaMemoryTypeHost ? static_cast<const double*>(at.devicePointer) : nullptr;
    }
    // dst32: the FP32 copy of the rows as well (width 4), or null
    void upload_cells(double* dst, const double* src, int width, float* dst32 = nullptr) {
        if (const double* hv = pinned_view(src)) {
            ck(launch_load_rows((int)N, width, perm_new.p, hv, dst, dst32, stream), "load rows");
            return;
        }
        const size_t bytes = (size_t)N * width * sizeof(double);
        ck(cudaMemcpyAsync(staging.p, src, bytes, cudaMemcpyHostToDevice, stream), "H2D");
        ck(launch_permute_rows((int)N, width, perm_old.p, staging.p, dst, false, stream), "permute");
        if (dst32) ck(launch_to_f32((size_t)N * width, dst, dst32, stream), "FP32 copy");
    }
    void download_cells(const double* src, double* dst, int width) {
        if (const double* hv = pinned_view(dst)) {
            ck(launch_store_rows((int)N, width, perm_new.p, src, const_cast<double*>(hv), stream), "store rows");
            ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
            return;
        }
        const size_t bytes = (size_t)N * width * sizeof(double);
        ck(launch_permute_rows((int)N, width, perm_old.p, src, staging.p, true, stream), "permute");
        ck(cudaMemcpyAsync(dst, staging.p, bytes, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }

    void build();
    void build_lsq_on_device(const TenoTables& t);
    double build_s[7] = {0, 0, 0, 0, 0, 0, 0};  // mgpu_build_times
};

namespace mgpu {

template <class F>
inline int guarded(F&& fn) {
    try {
        return fn();
    } catch (const CudaFail& e) {
        set_error(e.what());
        return MGPU_ERR_CUDA;
    } catch (const ArgFail& e) {
        set_error(e.what());
        return MGPU_ERR_ARG;
    } catch (const Unsupported& e) {
        set_error(e.what());
        return MGPU_ERR_UNSUPPORTED;
    } catch (const std::bad_alloc&) {
        set_error("host allocation failed");
        return MGPU_ERR_HOST;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MGPU_ERR_HOST;
    }
}

inline int need_ready(const mgpu_ctx* ctx) {
    if (!ctx) {
        set_error("null context");
        return MGPU_ERR_ARG;
    }
    if (!ctx->finalized) {
        set_error("context not finalized (call mgpu_finalize after adding boundaries)");
        return MGPU_ERR_STATE;
    }
    return MGPU_OK;
}

}  // namespace mgpu
