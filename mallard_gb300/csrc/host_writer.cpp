// host_writer.cpp -- VTU output of the solution, asynchronous.
//
// The reference writes its [[write_data]] variables every `interval` steps
// (DataWriter::write / write_vtu, src/io/data_writer.cpp:77-244), after a
// full device-to-host copy of the state each step (solver.cpp:422-423).
// Here the file format is the same (VTK XML UnstructuredGrid, raw appended
// data: Float64 cell arrays, 3-component points, UInt32 connectivity and
// offsets, UInt8 cell types 7), but a write only snapshots the state on the
// device: on a copy stream ordered after the work queued so far, a
// permutation kernel copies the requested arrays in caller order into a
// device staging slot, and the solver's stream waits for that snapshot
// alone.  The device-to-host copy into pinned memory and the file write
// then overlap the following steps; a worker thread writes the files in
// order.  Two slots let one snapshot be copied while the previous file is
// written.

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "host_ctx.h"

namespace mgpu {
namespace {

// [[write_data]] variable names (common_typedef.h:36-48, solver.cpp:337-349)
const char* const VAR_NAMES[10] = {"RHO", "RHOU_X", "RHOU_Y", "RHOE", "U_X", "U_Y", "P", "T", "H", "CFL"};

}  // namespace

// The VTU file of one snapshot: cell arrays in caller order, [n_vars][n_cells].
void write_vtu_file(const std::string& path, const HostMesh& m, const std::vector<std::string>& names,
                    const double* data) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("DataWriter::write_vtu: Could not open file: " + path + ".");
    const uint32_t nc = m.n_cells, nn = m.n_nodes;
    const uint64_t len_conn = m.off_noc[nc];
    uint64_t off = 0;
    std::ostringstream h;
    h << "<?xml version=\"1.0\"?>\n";
    h << "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    h << "  <UnstructuredGrid>\n";
    h << "    <Piece NumberOfPoints=\"" << nn << "\" NumberOfCells=\"" << nc << "\">\n";
    h << "      <PointData>\n      </PointData>\n";
    h << "      <CellData>\n";
    for (const auto& nm : names) {
        h << "        <DataArray type=\"Float64\" Name=\"" << nm << "\" format=\"appended\" offset=\"" << off
          << "\">\n        </DataArray>\n";
        off += 4 + (uint64_t)nc * 8;
    }
    h << "      </CellData>\n";
    h << "      <Points>\n        <DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"appended\" offset=\""
      << off << "\">\n        </DataArray>\n      </Points>\n";
    off += 4 + (uint64_t)nn * 24;
    h << "      <Cells>\n";
    h << "        <DataArray type=\"UInt32\" Name=\"connectivity\" format=\"appended\" offset=\"" << off
      << "\">\n        </DataArray>\n";
    off += 4 + len_conn * 4;
    h << "        <DataArray type=\"UInt32\" Name=\"offsets\" format=\"appended\" offset=\"" << off
      << "\">\n        </DataArray>\n";
    off += 4 + (uint64_t)nc * 4;
    h << "        <DataArray type=\"UInt8\" Name=\"types\" format=\"appended\" offset=\"" << off
      << "\">\n        </DataArray>\n";
    h << "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n";
    h << "<AppendedData encoding=\"raw\">\n_";
    const std::string head = h.str();
    out.write(head.data(), (std::streamsize)head.size());
    // each block: a 4-byte byte count (little-endian), then the values
    auto block = [&](const void* p, uint64_t bytes) {
        const uint32_t b = (uint32_t)bytes;
        out.write(reinterpret_cast<const char*>(&b), 4);
        out.write(reinterpret_cast<const char*>(p), (std::streamsize)bytes);
    };
    for (size_t v = 0; v < names.size(); ++v) block(data + v * (size_t)nc, (uint64_t)nc * 8);
    std::vector<double> pts((size_t)nn * 3);
    for (uint32_t i = 0; i < nn; ++i) {
        pts[3 * (size_t)i] = m.node_coords[2 * (size_t)i];
        pts[3 * (size_t)i + 1] = m.node_coords[2 * (size_t)i + 1];
        pts[3 * (size_t)i + 2] = 0.0;
    }
    block(pts.data(), pts.size() * 8);
    block(m.noc.data(), len_conn * 4);
    block(m.off_noc.data() + 1, (uint64_t)nc * 4);
    std::vector<uint8_t> types(nc, 7);  // VTK_POLYGON
    block(types.data(), nc);
    out << "\n</AppendedData>\n</VTKFile>\n";
    if (!out) throw std::runtime_error("DataWriter::write_vtu: Could not write to file: " + path + ".");
}

}  // namespace mgpu

using namespace mgpu;

struct mgpu_writer {
    mgpu_ctx* ctx = nullptr;
    std::string prefix;
    std::vector<int> vars;  // indices into VAR_NAMES
    std::vector<std::string> names;
    uint32_t interval = 1;
    cudaStream_t copy = nullptr;
    struct Slot {
        DevArray<double> dev;
        double* host = nullptr;  // pinned: [n_vars][n_cells] + dt
        cudaEvent_t taken = nullptr, copied = nullptr;
        bool busy = false;
    } slot[2];
    int next = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    struct Job {
        int slot;
        uint32_t step;
    };
    std::deque<Job> jobs;
    bool stop = false;
    std::string error;

    void run() {
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !jobs.empty(); });
                if (jobs.empty()) return;
                j = jobs.front();
            }
            std::string err;
            try {
                Slot& s = slot[j.slot];
                const cudaError_t e = cudaEventSynchronize(s.copied);
                if (e != cudaSuccess) throw std::runtime_error(std::string("snapshot copy: ") + cudaGetErrorString(e));
                const uint32_t nc = ctx->mesh.n_cells;
                double* data = s.host;
                // CFL = dt x spectral radius, as Solver::calc_dt forms it (solver.cpp:720-742)
                const double dt = data[vars.size() * (size_t)nc];
                for (size_t v = 0; v < vars.size(); ++v)
                    if (vars[v] == 9)
                        for (uint32_t c = 0; c < nc; ++c) data[v * (size_t)nc + c] = dt * data[v * (size_t)nc + c];
                char num[16];
                std::snprintf(num, sizeof(num), "%06u", j.step);
                write_vtu_file(prefix + "_" + num + ".vtu", ctx->mesh, names, data);
            } catch (const std::exception& e) {
                err = e.what();
            }
            std::lock_guard<std::mutex> lk(mu);
            if (!err.empty() && error.empty()) error = err;
            slot[j.slot].busy = false;
            jobs.pop_front();
            cv.notify_all();
        }
    }

    void wait_idle() {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return jobs.empty(); });
    }

    ~mgpu_writer() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
        for (auto& s : slot) {
            if (s.host) cudaFreeHost(s.host);
            if (s.taken) cudaEventDestroy(s.taken);
            if (s.copied) cudaEventDestroy(s.copied);
        }
        if (copy) cudaStreamDestroy(copy);
    }
};

extern "C" {

int mgpu_writer_create(mgpu_ctx* ctx, const char* prefix, const char* variables, uint32_t interval,
                       mgpu_writer** out) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!prefix || !variables || !out) throw ArgFail("DataWriter: prefix, variables and output required.");
        if (interval == 0) throw ArgFail("DataWriter: interval must be positive.");
        std::unique_ptr<mgpu_writer> w(new mgpu_writer());
        w->ctx = ctx;
        w->prefix = prefix;
        w->interval = interval;
        std::stringstream ss(variables);
        std::string tok;
        while (std::getline(ss, tok, ',')) {
            const size_t a = tok.find_first_not_of(" \t"), b = tok.find_last_not_of(" \t");
            if (a == std::string::npos) continue;
            tok = tok.substr(a, b - a + 1);
            int idx = -1;
            for (int i = 0; i < 10; ++i)
                if (tok == VAR_NAMES[i]) idx = i;
            if (idx < 0) throw ArgFail("DataWriter: Unknown variable: " + tok + ".");
            w->vars.push_back(idx);
            w->names.push_back(tok);
        }
        if (w->vars.empty()) throw ArgFail("DataWriter: No variables specified.");
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        ck(cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking), "cudaStreamCreate");
        const size_t n = (size_t)ctx->N * w->vars.size() + 1;
        for (auto& s : w->slot) {
            s.dev.alloc(n);
            ck(cudaMallocHost(&s.host, n * sizeof(double)), "cudaMallocHost");
            ck(cudaEventCreateWithFlags(&s.taken, cudaEventDisableTiming), "cudaEventCreate");
            ck(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming), "cudaEventCreate");
        }
        mgpu_writer* raw = w.get();
        w->worker = std::thread([raw] { raw->run(); });
        *out = w.release();
        return MGPU_OK;
    });
}

int mgpu_writer_write(mgpu_writer* w, uint32_t step, int force) {
    if (!w) return MGPU_ERR_ARG;
    if (!(step % w->interval == 0 || force)) return MGPU_OK;
    return guarded([&] {
        mgpu_ctx* ctx = w->ctx;
        {
            std::lock_guard<std::mutex> lk(w->mu);
            if (!w->error.empty()) throw std::runtime_error(w->error);
        }
        // the slot must be free of its previous file
        mgpu_writer::Slot& s = w->slot[w->next];
        {
            std::unique_lock<std::mutex> lk(w->mu);
            w->cv.wait(lk, [&] { return !s.busy; });
            s.busy = true;
        }
        const int id = w->next;
        w->next ^= 1;
        // a failure before the job is queued gives the slot back
        struct Release {
            mgpu_writer* w;
            mgpu_writer::Slot* s;
            bool armed = true;
            ~Release() {
                if (!armed) return;
                std::lock_guard<std::mutex> lk(w->mu);
                s->busy = false;
                w->cv.notify_all();
            }
        } release{w, &s};
        // snapshot: the copy stream follows the solver's stream, and the
        // solver's stream waits only for the snapshot
        bool wants_prims = false;
        for (int k : w->vars) wants_prims = wants_prims || (k >= 4 && k < 9);
        if (wants_prims) ctx->refresh_prims();
        cudaEvent_t after = nullptr;
        ck(cudaEventCreateWithFlags(&after, cudaEventDisableTiming), "cudaEventCreate");
        ck(cudaEventRecord(after, ctx->stream), "cudaEventRecord");
        ck(cudaStreamWaitEvent(w->copy, after, 0), "cudaStreamWaitEvent");
        cudaEventDestroy(after);
        const size_t nc = ctx->N;
        for (size_t v = 0; v < w->vars.size(); ++v) {
            const int k = w->vars[v];
            const double* src = k < 4 ? ctx->U.p + k : (k < 9 ? ctx->prim.p + (k - 4) : ctx->rho_cell.p);
            const int stride = k < 4 ? 4 : (k < 9 ? 5 : 1);
            ck(launch_permute_column((int)nc, stride, ctx->perm_old.p, src, s.dev.p + v * nc, w->copy),
               "snapshot");
        }
        ck(cudaMemcpyAsync(s.dev.p + w->vars.size() * nc, ctx->dt_ptr(), sizeof(double), cudaMemcpyDeviceToDevice,
                           w->copy),
           "snapshot dt");
        ck(cudaEventRecord(s.taken, w->copy), "cudaEventRecord");
        ck(cudaStreamWaitEvent(ctx->stream, s.taken, 0), "cudaStreamWaitEvent");
        ck(cudaMemcpyAsync(s.host, s.dev.p, (w->vars.size() * nc + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                           w->copy),
           "snapshot D2H");
        ck(cudaEventRecord(s.copied, w->copy), "cudaEventRecord");
        {
            std::lock_guard<std::mutex> lk(w->mu);
            w->jobs.push_back({id, step});
        }
        release.armed = false;
        w->cv.notify_all();
        return MGPU_OK;
    });
}

int mgpu_writer_flush(mgpu_writer* w) {
    if (!w) return MGPU_ERR_ARG;
    w->wait_idle();
    std::lock_guard<std::mutex> lk(w->mu);
    if (!w->error.empty()) {
        set_error(w->error);
        return MGPU_ERR_HOST;
    }
    return MGPU_OK;
}

void mgpu_writer_destroy(mgpu_writer* w) {
    if (!w) return;
    w->wait_idle();
    delete w;
}

int mgpu_vtu_write(const mgpu_mesh_buf* mesh, const char* path, uint32_t n_vars, const char* const* names,
                   const double* data) {
    if (!mesh || !path || (n_vars && (!names || !data))) {
        set_error("mgpu_vtu_write: null argument");
        return MGPU_ERR_ARG;
    }
    try {
        std::vector<std::string> nm;
        for (uint32_t i = 0; i < n_vars; ++i) nm.emplace_back(names[i]);
        write_vtu_file(path, mesh->m, nm, data);
        return MGPU_OK;
    } catch (const std::exception& e) {
        set_error(e.what());
        return MGPU_ERR_HOST;
    }
}

}  // extern "C"
