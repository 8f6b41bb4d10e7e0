// nw_writer.cu — trajectory frames off the step's critical path
// (include/nwgb.h, "trajectory output").
//
// The reference writes a frame synchronously: a blocking device-to-host copy
// of positions and velocities, then text formatting on the simulation thread
// (ParticleSystem::writeOutputs, simulation/particleSystem.cpp:481-532).
// Here a frame costs the step loop one device-to-device snapshot on the
// system's stream (HBM bandwidth); the copy to pinned host memory runs on the
// writer's own stream and the formatting on a writer thread, with two
// snapshot slots in flight.
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>

#include "nw_system.h"

namespace {

struct Slot {
    float4 *dpos = nullptr, *dvel = nullptr;  // device snapshot
    float4 *hpos = nullptr, *hvel = nullptr;  // pinned host copy
    cudaEvent_t snap = nullptr, done = nullptr;
    bool busy = false;
    int iteration = 0;
    float dt = 0.f;
    NwConfig cfg;
};

nw_status st_of(cudaError_t e)
{
    if (e == cudaSuccess) return NW_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? NW_ERR_NOMEM : NW_ERR_CUDA;
}

// One float as a C++ ostream prints it by default (%g, 6 significant digits).
void put_g(std::string& s, double x)
{
    char b[32];
    const int n = std::snprintf(b, sizeof(b), "%g", x);
    s.append(b, (size_t)n);
}

void put_u(std::string& s, unsigned long long x)
{
    char b[32];
    const int n = std::snprintf(b, sizeof(b), "%llu", x);
    s.append(b, (size_t)n);
}

void put_i(std::string& s, long long x)
{
    char b[32];
    const int n = std::snprintf(b, sizeof(b), "%lld", x);
    s.append(b, (size_t)n);
}

// The parameter line of a frame: the reference's keys
// (simulation/particleSystem.cpp:492-518) filled from the configuration.
std::string header_json(const NwConfig& c, int iteration, float dt, uint32_t nb, uint32_t ncells)
{
    std::string s = "{\"iteration\":";
    put_i(s, iteration);
    s += ",\"dt\":";
    put_g(s, dt);
    s += ",\"time\":";
    put_g(s, (float)iteration * dt);
    s += ",\"num_particles\":";
    put_u(s, nb);
    s += ",\"num_filaments\":";
    put_u(s, c.num_filaments);
    s += ",\"filament_size\":";
    put_u(s, c.filament_size);
    s += ",\"bond_spring_coef\":";
    put_g(s, c.bond_k);
    s += ",\"bond_spring_length\":";
    put_g(s, c.bond_r0);
    s += ",\"bond_bending_coef\":";
    put_g(s, c.bend_k);
    s += ",\"activity\":";
    put_g(s, c.activity);
    s += ",\"kbT\":";
    put_g(s, c.kT);
    s += ",\"gamma\":";
    put_g(s, c.gamma);
    s += ",\"particle_radius\":";
    put_g(s, c.radius);
    s += ",\"particle_mass\":";
    put_g(s, c.mass);
    s += ",\"num_cells\":";
    put_u(s, ncells);
    const char* vec[3] = {",\"grid_size\":[", ",\"box_size\":[", ",\"cell_size\":["};
    for (int k = 0; k < 3; ++k) {
        s += vec[k];
        for (int a = 0; a < 3; ++a) {
            if (a) s += ",";
            if (k == 0) put_u(s, c.grid[a]);
            else put_g(s, k == 1 ? c.box[a] : c.cell_size[a]);
        }
        s += "]";
    }
    s += ",\"boundaries\":[";
    for (int a = 0; a < 3; ++a) {
        if (a) s += ",";
        put_i(s, c.boundary[a]);
    }
    s += "],\"reverse_probability\":";
    put_g(s, c.reverse_probability);
    s += ",\"collision_spring_coef\":";
    put_g(s, c.spring);
    s += ",\"collision_damping_coef\":";
    put_g(s, c.damping);
    s += ",\"collision_shear_coef\":";
    put_g(s, c.shear);
    s += ",\"collision_attraction_coef\":";
    put_g(s, c.attraction);
    s += ",\"boundary_damping_coef\":";
    put_g(s, c.boundary_damping);
    s += "}\n";
    return s;
}

}  // namespace

struct nw_writer {
    nw_system* sys = nullptr;
    FILE* f = nullptr;
    cudaStream_t copy = nullptr;
    Slot slot[2];
    int next = 0;
    std::thread th;
    std::mutex m;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false;
    nw_status err = NW_OK;
    uint32_t n = 0, nb = 0;
};

namespace {

void write_slot(nw_writer* w, Slot& sl)
{
    std::string s;
    s.reserve((size_t)w->n * 64 + 1024);
    put_u(s, w->n);
    s += "\n";
    s += header_json(sl.cfg, sl.iteration, sl.dt, w->nb, w->sys->ncells);
    for (uint32_t i = 0; i < w->n; ++i) {
        const float4 p = sl.hpos[i], v = sl.hvel[i];
        s += i < w->nb ? "A " : "B ";
        put_g(s, p.x);
        s += " ";
        put_g(s, p.y);
        s += " ";
        put_g(s, p.z);
        s += " ";
        put_g(s, v.x);
        s += " ";
        put_g(s, v.y);
        s += " ";
        put_g(s, v.z);
        s += "\n";
        if (s.size() > (64u << 20)) {
            if (std::fwrite(s.data(), 1, s.size(), w->f) != s.size()) w->err = NW_ERR_IO;
            s.clear();
        }
    }
    if (std::fwrite(s.data(), 1, s.size(), w->f) != s.size()) w->err = NW_ERR_IO;
}

void writer_loop(nw_writer* w)
{
    cudaSetDevice(w->sys->device);
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(w->m);
            w->cv.wait(lk, [&] { return w->stop || !w->queue.empty(); });
            if (w->queue.empty()) return;
            k = w->queue.front();
        }
        Slot& sl = w->slot[k];
        const cudaError_t e = cudaEventSynchronize(sl.done);
        if (e == cudaSuccess) write_slot(w, sl);
        std::lock_guard<std::mutex> lk(w->m);
        if (e != cudaSuccess) w->err = st_of(e);
        w->queue.pop_front();
        sl.busy = false;
        w->cv.notify_all();
    }
}

}  // namespace

extern "C" {

nw_status nw_writer_open(nw_system* sys, const char* path, int append, nw_writer** out)
{
    if (!out) return NW_ERR_INVALID;
    *out = nullptr;
    if (!sys || !path) return NW_ERR_INVALID;
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return NW_ERR_IO;
    nw_writer* w = new nw_writer();
    w->sys = sys;
    w->f = f;
    w->nb = sys->nb;
    w->n = sys->nb + sys->ns;
    nw_status st = st_of(cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking));
    const size_t bytes = (size_t)(w->n ? w->n : 1) * sizeof(float4);
    for (int k = 0; k < 2 && st == NW_OK; ++k) {
        Slot& sl = w->slot[k];
        st = st_of(cudaMalloc(&sl.dpos, bytes));
        if (st == NW_OK) st = st_of(cudaMalloc(&sl.dvel, bytes));
        if (st == NW_OK) st = st_of(cudaMallocHost(&sl.hpos, bytes));
        if (st == NW_OK) st = st_of(cudaMallocHost(&sl.hvel, bytes));
        if (st == NW_OK) st = st_of(cudaEventCreateWithFlags(&sl.snap, cudaEventDisableTiming));
        if (st == NW_OK) st = st_of(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    }
    if (st != NW_OK) {
        nw_writer_close(w);
        return st;
    }
    w->th = std::thread(writer_loop, w);
    *out = w;
    return NW_OK;
}

nw_status nw_writer_frame(nw_writer* w, int iteration, float dt)
{
    if (!w) return NW_ERR_INVALID;
    nw_system* s = w->sys;
    Slot& sl = w->slot[w->next];
    {
        std::unique_lock<std::mutex> lk(w->m);
        w->cv.wait(lk, [&] { return !sl.busy; });
        if (w->err != NW_OK) return w->err;
    }
    // the state after the last update: beads in the current bead buffer,
    // solvent in the current solvent buffer
    const uint32_t cur = s->lists ? (uint32_t)((s->step + 1ull) & 1ull) : 0u;
    const nw::StepBuffers& B = s->B;
    const size_t bb = (size_t)s->nb * sizeof(float4), sb = (size_t)s->ns * sizeof(float4);
    cudaError_t e = cudaSuccess;
    if (bb) e = cudaMemcpyAsync(sl.dpos, B.pos2[cur], bb, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess && bb) e = cudaMemcpyAsync(sl.dvel, B.vel2[cur], bb, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess && sb)
        e = cudaMemcpyAsync(sl.dpos + s->nb, B.spos2[s->scur], sb, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess && sb)
        e = cudaMemcpyAsync(sl.dvel + s->nb, B.svel2[s->scur], sb, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.snap, s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(w->copy, sl.snap, 0);
    const size_t nbytes = (size_t)w->n * sizeof(float4);
    if (e == cudaSuccess && nbytes) e = cudaMemcpyAsync(sl.hpos, sl.dpos, nbytes, cudaMemcpyDeviceToHost, w->copy);
    if (e == cudaSuccess && nbytes) e = cudaMemcpyAsync(sl.hvel, sl.dvel, nbytes, cudaMemcpyDeviceToHost, w->copy);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, w->copy);
    if (e != cudaSuccess) return st_of(e);
    {
        std::lock_guard<std::mutex> lk(w->m);
        sl.busy = true;
        sl.iteration = iteration;
        sl.dt = dt;
        sl.cfg = s->cfg;
        w->queue.push_back(w->next);
    }
    w->cv.notify_all();
    w->next ^= 1;
    return NW_OK;
}

nw_status nw_writer_flush(nw_writer* w)
{
    if (!w) return NW_ERR_INVALID;
    std::unique_lock<std::mutex> lk(w->m);
    w->cv.wait(lk, [&] { return w->queue.empty(); });
    if (w->f && std::fflush(w->f) != 0 && w->err == NW_OK) w->err = NW_ERR_IO;
    return w->err;
}

nw_status nw_writer_close(nw_writer* w)
{
    if (!w) return NW_ERR_INVALID;
    nw_status st = NW_OK;
    if (w->th.joinable()) {
        st = nw_writer_flush(w);
        {
            std::lock_guard<std::mutex> lk(w->m);
            w->stop = true;
        }
        w->cv.notify_all();
        w->th.join();
    }
    if (w->copy) cudaStreamSynchronize(w->copy);
    for (auto& sl : w->slot) {
        cudaFree(sl.dpos);
        cudaFree(sl.dvel);
        cudaFreeHost(sl.hpos);
        cudaFreeHost(sl.hvel);
        if (sl.snap) cudaEventDestroy(sl.snap);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (w->copy) cudaStreamDestroy(w->copy);
    if (w->f) std::fclose(w->f);
    delete w;
    return st;
}

}  // extern "C"
