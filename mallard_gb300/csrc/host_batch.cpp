// host_batch.cpp -- the batched form behind the C ABI: many independent
// cases on a few meshes, stepped together by one launch per kernel.
//
// No counterpart in the reference (which runs one case per process).  Each
// distinct mesh gets one finalized solver context: its TENO tables and face
// geometry are built once and shared by all cases on that mesh.  The state
// of every case lives in batch-owned arrays whose rows are interleaved per
// 8-row tile (row(c) = ubase + ((c / 8) C + case) 8 + c % 8), so the warps
// working on one mesh tile for consecutive cases read the same table tile.
// Every case has its own time step, time and status flags.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "host_ctx.h"

using namespace mgpu;

struct mgpu_batch {
    mgpu_config cfg{};
    std::vector<BcHost> bcs;
    std::vector<const mgpu_mesh*> meshes;
    std::vector<uint32_t> C;
    std::vector<std::unique_ptr<mgpu_ctx, void (*)(mgpu_ctx*)>> groups;
    uint32_t n_cases = 0;
    bool finalized = false;
    cudaStream_t stream = nullptr, stream_owned = nullptr;  // launch stream; the batch's own
    BatchLaunch bl{};
    DevArray<double> U, Ut, W, prim, snd, G, dt, t;
    DevArray<float> fv, U32, Ut32;
    DevArray<unsigned long long> rmax;
    DevArray<unsigned> flags;
    DevArray<TenoArgs> d_teno;
    DevArray<FluxArgs> d_flux;
    DevArray<UpdateArgs> d_upd;
    DevArray<SpecArgs> d_spec;
    int teno_shape = 0, teno_blocks_per_sm = 0;  // autotuned launch of the reconstruction
    // per case: the steps left its FP64 primitives behind (they are recovered
    // from U when mgpu_batch_get_state asks for them)
    std::vector<uint8_t> prim_stale;
    cudaGraphExec_t exec = nullptr;
    double exec_cfl = -1.0;
    ~mgpu_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        cudaStream_t own = stream_owned ? stream_owned : stream;
        if (own) cudaStreamDestroy(own);
    }
};

namespace {

void destroy_ctx(mgpu_ctx* c) { mgpu_destroy(c); }

int need_batch(const mgpu_batch* b) {
    if (!b) {
        set_error("null batch");
        return MGPU_ERR_ARG;
    }
    if (!b->finalized) {
        set_error("batch not finalized (call mgpu_batch_finalize after adding boundaries)");
        return MGPU_ERR_STATE;
    }
    return MGPU_OK;
}

void batch_step(mgpu_batch* b, double cfl) {
    mgpu_ctx& g0 = *b->groups[0];
    ck(cudaMemsetAsync(b->rmax.p, 0, b->rmax.bytes(), b->stream), "cudaMemsetAsync");
    ck(launch_spectral_batch(b->bl, b->stream), "spectral");
    ck(launch_dt_batch(b->bl, (int)b->n_cases, cfl, b->stream), "dt");
    for (int k = 1; k <= 3; ++k) {
        const double* in = k == 1 ? b->U.p : b->Ut.p;
        const float* in32 = k == 1 ? b->U32.p : b->Ut32.p;
        ck(f32::launch_teno_batch(b->bl, in32, b->teno_shape, b->teno_blocks_per_sm, b->stream), "reconstruction");
        ck(f32::launch_flux_batch(b->bl, g0.gas, g0.bct, b->cfg.riemann_solver, g0.nq, in, b->stream), "flux");
        ck(launch_update_batch(b->bl, g0.gas, k, b->stream), "update");
    }
}

void check_case(const mgpu_batch* b, uint32_t group, uint32_t cs) {
    if (group >= b->groups.size() || cs >= b->C[group]) throw ArgFail("case out of range");
}

}  // namespace

extern "C" {

int mgpu_batch_create(uint32_t n_groups, const mgpu_mesh* const* meshes, const uint32_t* cases_per_group,
                      const mgpu_config* cfg, mgpu_batch** out) {
    if (!out) {
        set_error("null argument");
        return MGPU_ERR_ARG;
    }
    *out = nullptr;
    return guarded([&] {
        if (!meshes || !cases_per_group || !cfg) throw ArgFail("null argument");
        if (n_groups == 0 || n_groups > (uint32_t)MAX_GROUPS) throw ArgFail("1 to 8 mesh groups");
        if (cfg->precision != MGPU_PREC_FP32 || cfg->recon != MGPU_RECON_TENO || cfg->poly_order != 3 ||
            cfg->teno_variant == MGPU_TENO_REFERENCE)
            throw Unsupported("the batched form runs the FP32 form of corrected or robust TENO at p = 3");
        if (cfg->time_integrator != MGPU_INTEGRATOR_SSPRK3) throw Unsupported("the batched form integrates with SSPRK3");
        if (cfg->viscous) throw Unsupported("the batched form is inviscid");
        std::unique_ptr<mgpu_batch> b(new mgpu_batch());
        b->cfg = *cfg;
        for (uint32_t g = 0; g < n_groups; ++g) {
            if (!meshes[g] || cases_per_group[g] == 0) throw ArgFail("every group needs a mesh and a case");
            b->meshes.push_back(meshes[g]);
            b->C.push_back(cases_per_group[g]);
            b->n_cases += cases_per_group[g];
        }
        *out = b.release();
        return MGPU_OK;
    });
}

int mgpu_batch_add_boundary(mgpu_batch* b, uint32_t zone, int type, const double* data, int n_data) {
    if (!b) {
        set_error("null batch");
        return MGPU_ERR_ARG;
    }
    return guarded([&] {
        if (b->finalized) throw ArgFail("batch already finalized");
        BcHost h{};
        h.zone = zone;
        h.type = type;
        if (n_data < 0 || n_data > 6 || (n_data && !data)) throw ArgFail("boundary data: 0 to 6 values");
        for (int i = 0; i < n_data; ++i) h.data[i] = data[i];
        b->bcs.push_back(h);
        return MGPU_OK;
    });
}

int mgpu_batch_finalize(mgpu_batch* b) {
    if (!b) {
        set_error("null batch");
        return MGPU_ERR_ARG;
    }
    return guarded([&] {
        if (b->finalized) throw ArgFail("batch already finalized");
        ck(cudaSetDevice(b->cfg.device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        std::vector<TenoArgs> ht;
        std::vector<FluxArgs> hf;
        std::vector<UpdateArgs> hu;
        std::vector<SpecArgs> hs;
        BatchLaunch& bl = b->bl;
        bl.n_groups = (int)b->meshes.size();
        unsigned long long rows = 0, frows = 0;
        long long cell_t = 0, teno_t = 0, face_t = 0;
        unsigned case0 = 0;
        for (size_t g = 0; g < b->meshes.size(); ++g) {
            mgpu_ctx* c = nullptr;
            mgpu_config cfg = b->cfg;
            if (mgpu_create(b->meshes[g], &cfg, &c) != MGPU_OK) throw ArgFail(mgpu_last_error());
            b->groups.emplace_back(c, destroy_ctx);
            for (const BcHost& h : b->bcs) {
                int nd = h.type == MGPU_BC_UPT ? 4 : (h.type == MGPU_BC_P_OUT ? 1 : 0);
                if (mgpu_add_boundary(c, h.zone, h.type, nd ? h.data : nullptr, nd) != MGPU_OK)
                    throw ArgFail(mgpu_last_error());
            }
            if (mgpu_finalize(c) != MGPU_OK) throw ArgFail(mgpu_last_error());
            const unsigned Cg = b->C[g];
            const unsigned long long npad = (c->N + 7ull) / 8 * 8, fpad = (c->F_real + 7ull) / 8 * 8;
            bl.C[g] = Cg;
            bl.case0[g] = case0;
            bl.n_cells[g] = (int)c->N;
            bl.n_faces[g] = (int)c->F_flux;
            bl.ubase[g] = rows;
            bl.fbase[g] = frows;
            bl.cell0[g] = cell_t;
            bl.teno0[g] = teno_t;
            bl.face0[g] = face_t;
            rows += npad * Cg;
            frows += fpad * Cg;
            cell_t += (long long)((npad * Cg + 31) / 32 * 32);  // whole warps per group
            teno_t += (long long)(npad * Cg * 4);
            face_t += (long long)(((c->F_flux + 7ull) / 8 * 8) * Cg);
            case0 += Cg;
            ht.push_back(c->teno);
            FluxArgs fa{};
            fa.n_faces = (int)c->F_flux;
            fa.lr = c->lr.p;
            fa.nrm = c->nrm.p;
            fa.nrm32 = c->nrm32.p;
            fa.area = c->area.p;
            fa.bc = c->bcidx.p;
            fa.guard = c->cfg.teno_variant == MGPU_TENO_ROBUST;
            for (int i = 0; i < 4; ++i) {
                fa.qw[i] = c->qw[i];
                fa.qw_f[i] = (float)c->qw[i];
            }
            hf.push_back(fa);
            hu.push_back(c->update_args());
            SpecArgs sa{};
            sa.n_cells = (int)c->N;
            sa.cfaces = c->cfaces.p;
            sa.lr = c->lr.p;
            sa.nrm = c->nrm.p;
            sa.dxn = c->dxn.p;
            c->spec_fp32(sa);  // gas constants; the state rows are the batch's (below)
            hs.push_back(sa);
            if (c->nq != b->groups[0]->nq) throw Unsupported("all meshes need the same face quadrature");
        }
        bl.cell0[bl.n_groups] = cell_t;
        bl.teno0[bl.n_groups] = teno_t;
        bl.face0[bl.n_groups] = face_t;
        const int nq = b->groups[0]->nq;
        b->U.alloc(rows * 4);
        b->Ut.alloc(rows * 4);
        b->W.alloc(rows * 4);
        b->prim.alloc(rows * 5);
        b->U32.alloc(rows * 4);
        b->Ut32.alloc(rows * 4);
        b->snd.alloc(rows);
        b->fv.alloc(frows * nq * 8);
        b->G.alloc(frows * 4);
        b->dt.alloc(b->n_cases);
        b->t.alloc(b->n_cases);
        b->rmax.alloc(b->n_cases);
        b->flags.alloc(b->n_cases);
        b->d_teno.upload(ht);
        b->d_flux.upload(hf);
        b->d_upd.upload(hu);
        for (SpecArgs& sa : hs) sa.u32 = reinterpret_cast<const float4*>(b->U32.p);
        b->d_spec.upload(hs);
        bl.teno = b->d_teno.p;
        bl.flux = b->d_flux.p;
        bl.upd = b->d_upd.p;
        bl.spec = b->d_spec.p;
        bl.U = b->U.p;
        bl.Ut = b->Ut.p;
        bl.W = b->W.p;
        bl.prim = b->prim.p;
        bl.U32 = b->U32.p;
        bl.Ut32 = b->Ut32.p;
        bl.snd = b->snd.p;
        bl.G = b->G.p;
        bl.fv = b->fv.p;
        bl.dt = b->dt.p;
        bl.t = b->t.p;
        bl.rmax = b->rmax.p;
        bl.flags = b->flags.p;
        b->prim_stale.assign(b->n_cases, 0);
        b->finalized = true;
        return MGPU_OK;
    });
}

void mgpu_batch_destroy(mgpu_batch* b) { delete b; }

uint32_t mgpu_batch_n_cases(const mgpu_batch* b) { return b ? b->n_cases : 0; }

int mgpu_batch_set_state(mgpu_batch* b, uint32_t group, uint32_t cs, const double* Uh, const double* primh) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        if (!Uh) throw ArgFail("null state");
        check_case(b, group, cs);
        mgpu_ctx& c = *b->groups[group];
        const size_t bytes = (size_t)c.N * 4 * sizeof(double);
        ck(cudaMemcpyAsync(c.staging.p, Uh, bytes, cudaMemcpyHostToDevice, b->stream), "H2D");
        ck(launch_batch_rows((int)c.N, 4, c.perm_old.p, c.staging.p, b->U.p, b->bl.ubase[group], b->C[group], cs,
                             true, b->stream),
           "rows");
        ck(launch_batch_prims((int)c.N, c.gas, b->U.p, b->prim.p, b->snd.p, b->U32.p, b->bl.ubase[group], b->C[group],
                              cs, b->stream),
           "primitives");
        if (primh) {
            ck(cudaMemcpyAsync(c.staging.p, primh, (size_t)c.N * 5 * sizeof(double), cudaMemcpyHostToDevice,
                               b->stream),
               "H2D");
            ck(launch_batch_rows((int)c.N, 5, c.perm_old.p, c.staging.p, b->prim.p, b->bl.ubase[group], b->C[group],
                                 cs, true, b->stream),
               "rows");
        }
        const uint32_t gc = b->bl.case0[group] + cs;
        ck(cudaMemsetAsync(b->flags.p + gc, 0, sizeof(unsigned), b->stream), "cudaMemsetAsync");
        ck(cudaMemsetAsync(b->t.p + gc, 0, sizeof(double), b->stream), "cudaMemsetAsync");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        b->prim_stale[gc] = 0;
        return MGPU_OK;
    });
}

int mgpu_batch_get_state(mgpu_batch* b, uint32_t group, uint32_t cs, double* Uh, double* primh) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        check_case(b, group, cs);
        mgpu_ctx& c = *b->groups[group];
        if (Uh) {
            ck(launch_batch_rows((int)c.N, 4, c.perm_old.p, b->U.p, c.staging.p, b->bl.ubase[group], b->C[group], cs,
                                 false, b->stream),
               "rows");
            ck(cudaMemcpyAsync(Uh, c.staging.p, (size_t)c.N * 4 * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
               "D2H");
            ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        }
        if (primh) {
            const uint32_t gc = b->bl.case0[group] + cs;
            if (b->prim_stale[gc]) {
                ck(launch_batch_prims((int)c.N, c.gas, b->U.p, b->prim.p, b->snd.p, b->U32.p, b->bl.ubase[group],
                                      b->C[group], cs, b->stream),
                   "primitives");
                b->prim_stale[gc] = 0;
            }
            ck(launch_batch_rows((int)c.N, 5, c.perm_old.p, b->prim.p, c.staging.p, b->bl.ubase[group], b->C[group],
                                 cs, false, b->stream),
               "rows");
            ck(cudaMemcpyAsync(primh, c.staging.p, (size_t)c.N * 5 * sizeof(double), cudaMemcpyDeviceToHost,
                               b->stream),
               "D2H");
            ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        }
        return MGPU_OK;
    });
}

int mgpu_batch_run(mgpu_batch* b, double cfl, uint32_t n_steps) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        if (!b->exec || b->exec_cfl != cfl) {
            if (b->exec) {
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
            }
            cudaGraph_t g = nullptr;
            ck(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            try {
                batch_step(b, cfl);
            } catch (...) {
                cudaStreamEndCapture(b->stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            ck(cudaStreamEndCapture(b->stream, &g), "cudaStreamEndCapture");
            const cudaError_t e = cudaGraphInstantiate(&b->exec, g, 0);
            cudaGraphDestroy(g);
            ck(e, "cudaGraphInstantiate");
            b->exec_cfl = cfl;
        }
        if (n_steps > 0) std::fill(b->prim_stale.begin(), b->prim_stale.end(), 1);
        for (uint32_t s = 0; s < n_steps; ++s) ck(cudaGraphLaunch(b->exec, b->stream), "cudaGraphLaunch");
        return MGPU_OK;
    });
}

int mgpu_batch_set_stream(mgpu_batch* b, void* stream) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        if (stream) {
            // the batch launches on the caller's stream from now on
            b->stream_owned = b->stream_owned ? b->stream_owned : b->stream;
            b->stream = (cudaStream_t)stream;
        } else if (b->stream_owned) {
            b->stream = b->stream_owned;
        }
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        return MGPU_OK;
    });
}

int mgpu_batch_synchronize(mgpu_batch* b) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_batch_status(mgpu_batch* b, uint32_t* flags, double* times) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        if (flags)
            ck(cudaMemcpyAsync(flags, b->flags.p, b->n_cases * sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream),
               "D2H");
        if (times)
            ck(cudaMemcpyAsync(times, b->t.p, b->n_cases * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "D2H");
        ck(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_batch_set_launch_shape(mgpu_batch* b, int shape, int blocks_per_sm) {
    if (int rc = need_batch(b)) return rc;
    if (shape < 0 || shape >= f32::TENO32_BATCH_SHAPES || blocks_per_sm < 0) {
        set_error("launch shape out of range");
        return MGPU_ERR_ARG;
    }
    b->teno_shape = shape;
    b->teno_blocks_per_sm = blocks_per_sm;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return MGPU_OK;
}

int mgpu_batch_autotune(mgpu_batch* b, double* ms, int* shape, int* blocks_per_sm) {
    if (int rc = need_batch(b)) return rc;
    return guarded([&] {
        // launch shapes x persistent grid sizes (CTAs per SM; 0 = one thread per item)
        const int grids[4] = {0, 2, 4, 8};
        cudaEvent_t e0, e1;
        ck(cudaEventCreate(&e0), "cudaEventCreate");
        ck(cudaEventCreate(&e1), "cudaEventCreate");
        double best = 1e300;
        int bs = 0, bg = 0;
        for (int sh = 0; sh < f32::TENO32_BATCH_SHAPES; ++sh)
            for (int gi = 0; gi < 4; ++gi) {
                if (sh >= 4 && gi > 0) continue;  // the staged and resident shapes have one grid
                ck(f32::launch_teno_batch(b->bl, b->U32.p, sh, grids[gi], b->stream), "reconstruction");
                ck(cudaEventRecord(e0, b->stream), "cudaEventRecord");
                for (int r = 0; r < 3; ++r)
                    ck(f32::launch_teno_batch(b->bl, b->U32.p, sh, grids[gi], b->stream), "reconstruction");
                ck(cudaEventRecord(e1, b->stream), "cudaEventRecord");
                ck(cudaEventSynchronize(e1), "cudaEventSynchronize");
                float f = 0.f;
                ck(cudaEventElapsedTime(&f, e0, e1), "cudaEventElapsedTime");
                const double m = f / 3.0;
                if (ms) ms[sh * 4 + gi] = m;
                if (m < best) {
                    best = m;
                    bs = sh;
                    bg = grids[gi];
                }
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->teno_shape = bs;
        b->teno_blocks_per_sm = bg;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        if (shape) *shape = bs;
        if (blocks_per_sm) *blocks_per_sm = bg;
        return MGPU_OK;
    });
}

}  // extern "C"
