// Snapshots of the device state: GPLUM's snapNNNNNN.dat / snap_tmp.dat
// written from, and read into, the engine's HBM-resident bodies.
//
// Writing: the fields the file needs are copied device-to-host into pinned
// buffers on the library stream (so they are the state as of this point of
// the stream, whatever later phases do), an event marks the copies, and the
// file is formatted and written by p3t_snapshot_write_host -- on a host
// thread when async, so the next tree step overlaps the formatting and the
// disk write.  Reading: the file is parsed on the host and loaded with the
// start-up reset of GPLUM's main loop (src/main_p3t.cpp:238-305).
#include <cmath>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_engine.cuh"

namespace p3t {
namespace {

struct PinnedBodies {
    std::vector<void *> blocks;
    p3t_bodies_t b{};
    ~PinnedBodies() {
        for (void *p : blocks) cudaFreeHost(p);
    }
    template <class T>
    int alloc(T **p, size_t n) {
        void *q = nullptr;
        if (cudaMallocHost(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return ST_BAD_INDEX;
        blocks.push_back(q);
        *p = (T *)q;
        return 0;
    }
};

struct SnapJob {
    std::thread th;
    int status = 0;
    bool running = false;
};
SnapJob g_job;
std::mutex g_job_mu;

int join_job() {
    if (g_job.running) {
        g_job.th.join();
        g_job.running = false;
    }
    const int s = g_job.status;
    g_job.status = 0;
    return s;
}

}  // namespace
}  // namespace p3t

using namespace p3t;

extern "C" {

int p3t_snapshot_wait(void) {
    std::lock_guard<std::mutex> lk(g_job_mu);
    return join_job();
}

int p3t_snapshot_write(const char *path, int binary, const p3t_file_header_t *header, int async) {
    if (!path || !header) return P3T_IO_BAD_ARGUMENT;
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    std::lock_guard<std::mutex> lk(g_job_mu);
    int r = join_job();  // one write in flight at a time
    if (r) return r;
    const State &S = E.S;
    const int n = S.n;
    auto *pb = new PinnedBodies();
    p3t_bodies_t &b = pb->b;
    cudaStream_t st = E.c->stream;
    auto d2h_async = [&](auto *dst, const auto *src, size_t count) {
        return cuda_status(cudaMemcpyAsync(dst, src, count * sizeof(*dst), cudaMemcpyDeviceToHost, st));
    };
    // the ASCII fields, then (binary) every other FPGrav field the state carries
    if ((r = pb->alloc(&b.id, n)) || (r = pb->alloc(&b.mass, n)) || (r = pb->alloc(&b.r_planet, n)) ||
        (r = pb->alloc(&b.f, n)) || (r = pb->alloc(&b.pos, 3 * (size_t)n)) || (r = pb->alloc(&b.vel, 3 * (size_t)n)) ||
        (r = pb->alloc(&b.number, n))) {
        delete pb;
        return r;
    }
    static_assert(sizeof(long long) == sizeof(int64_t), "id width");
    r = d2h_async(b.id, (const long long *)S.id, n);
    if (!r) r = d2h_async(b.mass, S.mass, n);
    if (!r) r = d2h_async(b.r_planet, S.r_planet, n);
    if (!r) r = d2h_async(b.f, S.f, n);
    if (!r) r = d2h_async(b.pos, S.pos, 3 * (size_t)n);
    if (!r) r = d2h_async(b.vel, S.vel, 3 * (size_t)n);
    if (!r) r = d2h_async(b.number, S.number, n);
    if (!r && binary) {
        struct V {
            double **h;
            const double *d;
            size_t w;
        };
        const V vs[] = {{&b.acc, S.acc, 3},       {&b.acc_d, S.acc_d, 3},   {&b.jerk_d, S.jerk_d, 3},
                        {&b.acc_s, S.acc_s, 3},   {&b.jerk_s, S.jerk_s, 3}, {&b.phi, S.phi, 1},
                        {&b.phi_d, S.phi_d, 1},   {&b.phi_s, S.phi_s, 1},   {&b.r_out, S.r_out, 1},
                        {&b.r_search, S.r_search, 1}, {&b.r_out_inv, S.r_out_inv, 1}, {&b.v_disp, S.v_disp, 1},
                        {&b.time, S.time, 1},     {&b.dt, S.dt, 1},         {&b.acc0, S.acc0, 1}};
        for (const V &v : vs) {
            if ((r = pb->alloc(v.h, v.w * n)) || (r = d2h_async(*v.h, v.d, v.w * n))) break;
        }
        struct I {
            int **h;
            const int32_t *d;
        };
        const I is[] = {{&b.rank, S.rank},           {&b.id_max, S.id_max}, {&b.id_min, S.id_min},
                        {&b.n_cluster, S.n_cluster}, {&b.dead, S.dead},     {&b.merged, S.merged}};
        for (const I &v : is) {
            if (r) break;
            if ((r = pb->alloc(v.h, n)) || (r = d2h_async(*v.h, (const int *)v.d, n))) break;
        }
        if (!r && !(r = pb->alloc(&b.id_cluster, n))) r = d2h_async(b.id_cluster, (const long long *)S.id_cluster, n);
    }
    cudaEvent_t ev = nullptr;
    if (!r) r = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    if (!r) r = cuda_status(cudaEventRecord(ev, st));
    if (r) {
        if (ev) cudaEventDestroy(ev);
        cudaStreamSynchronize(st);
        delete pb;
        return r;
    }
    p3t_file_header_t h = *header;
    h.n_body = n;
    std::string file(path);
    auto job = [pb, ev, h, file, binary, n]() -> int {
        int s = cuda_status(cudaEventSynchronize(ev));
        cudaEventDestroy(ev);
        if (!s) s = p3t_snapshot_write_host(file.c_str(), binary, &h, n, &pb->b);
        delete pb;
        return s;
    };
    if (!async) return job();
    g_job.running = true;
    g_job.status = 0;
    g_job.th = std::thread([job]() { g_job.status = job(); });
    return 0;
}

int p3t_snapshot_read(const char *path, int binary, p3t_file_header_t *header) {
    if (!path || !header) return P3T_IO_BAD_ARGUMENT;
    Engine &E = g_eng;
    if (!E.c && !(E.c = ctx_get(0))) return -(int)cudaErrorNoDevice;
    const int n = p3t_snapshot_read_host(path, binary, header, 0, nullptr);
    if (n < 0) return n;
    std::vector<long long> id(n), id_cluster(binary ? n : 0);
    std::vector<double> mass(n), r_planet(n), f(n), pos(3 * (size_t)n), vel(3 * (size_t)n);
    std::vector<double> v3[5], s1[7];
    std::vector<int> i1[3];
    p3t_bodies_t b{};
    b.id = id.data();
    b.mass = mass.data();
    b.r_planet = r_planet.data();
    b.f = f.data();
    b.pos = pos.data();
    b.vel = vel.data();
    double **v3p[5] = {&b.acc, &b.acc_d, &b.jerk_d, &b.acc_s, &b.jerk_s};
    double **s1p[7] = {&b.phi, &b.phi_d, &b.phi_s, &b.v_disp, &b.dt, &b.acc0, &b.time};
    int **i1p[3] = {&b.rank, &b.id_max, &b.id_min};
    if (binary) {
        for (int k = 0; k < 5; k++) {
            v3[k].assign(3 * (size_t)n, 0.);
            *v3p[k] = v3[k].data();
        }
        for (int k = 0; k < 7; k++) {
            s1[k].assign(n, 0.);
            *s1p[k] = s1[k].data();
        }
        for (int k = 0; k < 3; k++) {
            i1[k].assign(n, 0);
            *i1p[k] = i1[k].data();
        }
        b.id_cluster = id_cluster.data();
    }
    int r = p3t_snapshot_read_host(path, binary, header, n, &b);
    if (r < 0) return r;
    // src/main_p3t.cpp:301-302: a missing radius comes from the mass
    // (FPGrav::setRPlanet, src/particle.h:757-759), a missing increase
    // factor is FPGrav::increase_factor (1 unless parameter.dat sets f)
    const double dens = E.c->params[20];
    for (int i = 0; i < n; i++) {
        if (r_planet[i] <= 0.) r_planet[i] = std::pow(0.75 * mass[i] / (3.14159265358979323846 * dens), 1. / 3.);
        if (f[i] == 0.) f[i] = 1.;
    }
    if ((r = E.load(n, id.data(), mass.data(), r_planet.data(), f.data(), pos.data(), vel.data()))) return r;
    State &S = E.S;
    cudaStream_t st = E.c->stream;
    if (binary) {
        double *dv[5] = {S.acc, S.acc_d, S.jerk_d, S.acc_s, S.jerk_s};
        for (int k = 0; k < 5; k++)
            if ((r = cuda_status(cudaMemcpyAsync(dv[k], v3[k].data(), 3 * (size_t)n * sizeof(double),
                                                 cudaMemcpyHostToDevice, st))))
                return r;
        // time is reset below; the hard-part state carries over
        double *ds[6] = {S.phi, S.phi_d, S.phi_s, S.v_disp, S.dt, S.acc0};
        for (int k = 0; k < 6; k++)
            if ((r = cuda_status(cudaMemcpyAsync(ds[k], s1[k].data(), (size_t)n * sizeof(double),
                                                 cudaMemcpyHostToDevice, st))))
                return r;
        int32_t *di[3] = {S.rank, S.id_max, S.id_min};
        for (int k = 0; k < 3; k++)
            if ((r = cuda_status(cudaMemcpyAsync(di[k], i1[k].data(), (size_t)n * sizeof(int),
                                                 cudaMemcpyHostToDevice, st))))
                return r;
        if ((r = cuda_status(cudaMemcpyAsync(S.id_cluster, id_cluster.data(), (size_t)n * sizeof(long long),
                                             cudaMemcpyHostToDevice, st))))
            return r;
    }
    // every body's time is the run's time (src/main_p3t.cpp:296)
    std::vector<double> t(n, header->time);
    if ((r = cuda_status(cudaMemcpyAsync(S.time, t.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st))) ||
        (r = cuda_status(cudaStreamSynchronize(st))))
        return r;
    // next id: max(header id_next - 1, largest id) + 1 (src/main_p3t.cpp:264,287-305)
    if ((long long)header->id_next > E.id_next) E.id_next = header->id_next;
    return n;
}

}  // extern "C"
