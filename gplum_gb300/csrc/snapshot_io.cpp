// GPLUM's snapshot files, written and read on the host.
//
// The formats are GPLUM's own (the restart and analysis tools of a GPLUM run
// read these files unchanged):
//   * ASCII snapshot snapNNNNNN.dat (makeSnap, src/func.h:53-66 of GPLUM):
//     one header line (FileHeader::writeAscii, src/energy.h:100-110:
//     "%g\t%d\t%d" then ten "%20.15e" -- time, n_body, id_next, and etot,
//     ekin, ephi_sun, ephi_planet, edisp of the initial and of the current
//     energy), then one line per body (FPGrav::writeAscii,
//     src/particle.h:845-858: id "%lld", mass, r_planet, f, pos, vel as
//     "%20.15e", neighbor.number and a flag word as "%d", tab-separated);
//   * binary restart file snap_tmp.dat (makeSnapTmp, src/func.h:68-80):
//     the FileHeader object (128 bytes) then every FPGrav object as it lies
//     in memory (src/particle.h:868-876) -- 344 bytes in the build with
//     individual cutoffs, quadrupole moments and collisions (the layout is
//     spelled out below and checked against GPLUM's compiled class);
//   * header, then the bodies in order: FDPS's writeParticleAscii /
//     writeParticleBinary on one process (FDPS is not part of GPLUM's tree;
//     this is its documented single-file behaviour).
// Reading accepts an ASCII file with or without the header line (GPLUM's
// initial-condition files, src/main_p3t.cpp:248-268) and the binary file.
// ASCII lines are formatted and parsed in parallel chunks (OpenMP) and
// written in order.
#include <algorithm>
#include <cerrno>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/gplum_p3t.h"
#include "p3t_fpgrav.h"

namespace {

using p3t::FPGravRecord;

// FileHeader (src/energy.h:65-71): n_body, id_next, time, two Energy objects
// of seven doubles (etot, ekin, ephi_sun, ephi_planet, ephi, ephi_d, edisp).
struct FileHeaderRecord {
    int32_t n_body, id_next;
    double time;
    double e_init[7], e_now[7];
};
static_assert(sizeof(FileHeaderRecord) == 128, "FileHeader record");

constexpr int CHUNK = 8192;  // bodies per formatting / parsing task

void fmt_header(std::string &s, const p3t_file_header_t *h) {
    char buf[512];
    const double *a = h->e_init, *b = h->e_now;
    // the five Energy fields the ASCII header carries: etot ekin ephi_sun ephi_planet edisp
    const int m = std::snprintf(buf, sizeof buf,
                                "%g\t%d\t%d\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t"
                                "%20.15e\t%20.15e\t%20.15e\n",
                                h->time, h->n_body, h->id_next, a[0], a[1], a[2], a[3], a[6], b[0], b[1], b[2], b[3],
                                b[6]);
    s.append(buf, (size_t)m);
}

void fmt_body(std::string &s, const p3t_bodies_t *b, int i) {
    char buf[512];
    const double *x = b->pos + 3 * (size_t)i, *v = b->vel + 3 * (size_t)i;
    const int m = std::snprintf(buf, sizeof buf,
                                "%lld\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e\t%20.15e"
                                "\t%d\t%d\n",
                                (long long)b->id[i], b->mass[i], b->r_planet[i], b->f[i], x[0], x[1], x[2], v[0], v[1],
                                v[2], b->number ? b->number[i] : 0, 0);
    s.append(buf, (size_t)m);
}

void to_record(FPGravRecord &r, const p3t_bodies_t *b, int i) {
    std::memset(&r, 0, sizeof r);
    auto v3 = [&](double *dst, const double *src) {
        if (src) std::memcpy(dst, src + 3 * (size_t)i, 3 * sizeof(double));
    };
    auto s1 = [&](const double *src) { return src ? src[i] : 0.; };
    auto i1 = [&](const int *src, int dflt) { return src ? src[i] : dflt; };
    r.id_local = i;
    r.myrank = 0;
    v3(r.pos, b->pos);
    r.r_out = s1(b->r_out);
    r.r_search = s1(b->r_search);
    r.id = b->id[i];
    r.mass = b->mass[i];
    v3(r.vel, b->vel);
    v3(r.acc_d, b->acc_d);
    v3(r.acc, b->acc);
    v3(r.acc_s, b->acc_s);
    v3(r.jerk_d, b->jerk_d);
    v3(r.jerk_s, b->jerk_s);
    r.phi = s1(b->phi);
    r.phi_d = s1(b->phi_d);
    r.phi_s = s1(b->phi_s);
    r.v_disp = s1(b->v_disp);
    r.r_out_inv = s1(b->r_out_inv);
    r.time = s1(b->time);
    r.dt = s1(b->dt);
    r.acc0 = s1(b->acc0);
    r.r_planet = s1(b->r_planet);
    r.f = s1(b->f);
    r.number = i1(b->number, 0);
    r.rank = i1(b->rank, 0);
    r.id_max = i1(b->id_max, -1);
    r.id_min = i1(b->id_min, 2147483646);  // NeighborInfo(): S32_MAX - 1
    r.id_cluster = b->id_cluster ? b->id_cluster[i] : b->id[i];
    r.n_cluster = i1(b->n_cluster, 0);
    r.in_domain = 1;
    r.is_sent = 0;
    r.is_dead = (uint8_t)(i1(b->dead, 0) != 0);
    r.is_merged = (uint8_t)(i1(b->merged, 0) != 0);
}

void from_record(const FPGravRecord &r, const p3t_bodies_t *b, int i) {
    auto v3 = [&](double *dst, const double *src) {
        if (dst) std::memcpy(dst + 3 * (size_t)i, src, 3 * sizeof(double));
    };
    auto s1 = [&](double *dst, double v) {
        if (dst) dst[i] = v;
    };
    auto i1 = [&](int *dst, int v) {
        if (dst) dst[i] = v;
    };
    if (b->id) b->id[i] = r.id;
    s1(b->mass, r.mass);
    v3(b->pos, r.pos);
    v3(b->vel, r.vel);
    v3(b->acc_d, r.acc_d);
    v3(b->acc, r.acc);
    v3(b->acc_s, r.acc_s);
    v3(b->jerk_d, r.jerk_d);
    v3(b->jerk_s, r.jerk_s);
    s1(b->r_out, r.r_out);
    s1(b->r_search, r.r_search);
    s1(b->phi, r.phi);
    s1(b->phi_d, r.phi_d);
    s1(b->phi_s, r.phi_s);
    s1(b->v_disp, r.v_disp);
    s1(b->r_out_inv, r.r_out_inv);
    s1(b->time, r.time);
    s1(b->dt, r.dt);
    s1(b->acc0, r.acc0);
    s1(b->r_planet, r.r_planet);
    s1(b->f, r.f);
    i1(b->number, r.number);
    i1(b->rank, r.rank);
    i1(b->id_max, r.id_max);
    i1(b->id_min, r.id_min);
    if (b->id_cluster) b->id_cluster[i] = r.id_cluster;
    i1(b->n_cluster, r.n_cluster);
    i1(b->dead, r.is_dead);
    i1(b->merged, r.is_merged);
}

int write_all(FILE *fp, const void *p, size_t bytes) {
    return std::fwrite(p, 1, bytes, fp) == bytes ? 0 : P3T_IO_ERROR;
}

// the next line of [p, end): returns its end (at '\n' or end)
const char *line_end(const char *p, const char *end) {
    const void *q = std::memchr(p, '\n', (size_t)(end - p));
    return q ? (const char *)q : end;
}

bool blank(const char *p, const char *e) {
    for (; p < e; p++)
        if (*p != ' ' && *p != '\t' && *p != '\r') return false;
    return true;
}

// one ASCII body line: id mass r_planet f x y z vx vy vz number flag
bool parse_body(const char *p, const char *e, const p3t_bodies_t *b, int i) {
    std::string line(p, (size_t)(e - p));
    const char *s = line.c_str();
    char *q = nullptr;
    errno = 0;
    const long long id = std::strtoll(s, &q, 10);
    if (q == s) return false;
    double v[9];
    for (int k = 0; k < 9; k++) {
        s = q;
        v[k] = std::strtod(s, &q);
        if (q == s) return false;
    }
    s = q;
    const long number = std::strtol(s, &q, 10);
    if (q == s) return false;
    if (b->id) b->id[i] = id;
    if (b->mass) b->mass[i] = v[0];
    if (b->r_planet) b->r_planet[i] = v[1];
    if (b->f) b->f[i] = v[2];
    if (b->pos) std::memcpy(b->pos + 3 * (size_t)i, v + 3, 3 * sizeof(double));
    if (b->vel) std::memcpy(b->vel + 3 * (size_t)i, v + 6, 3 * sizeof(double));
    if (b->number) b->number[i] = (int)number;
    return true;
}

bool parse_header(const char *p, const char *e, p3t_file_header_t *h) {
    std::string line(p, (size_t)(e - p));
    const char *s = line.c_str();
    char *q = nullptr;
    const double t = std::strtod(s, &q);
    if (q == s) return false;
    s = q;
    const long nb = std::strtol(s, &q, 10);
    if (q == s) return false;
    s = q;
    const long idn = std::strtol(s, &q, 10);
    if (q == s) return false;
    double v[10];
    for (int k = 0; k < 10; k++) {
        s = q;
        v[k] = std::strtod(s, &q);
        if (q == s) return false;
    }
    std::memset(h, 0, sizeof *h);
    h->time = t;
    h->n_body = (int)nb;
    h->id_next = (int)idn;
    const int idx[5] = {0, 1, 2, 3, 6};
    for (int k = 0; k < 5; k++) {
        h->e_init[idx[k]] = v[k];
        h->e_now[idx[k]] = v[5 + k];
    }
    return true;
}

}  // namespace

extern "C" {

int p3t_snapshot_write_host(const char *path, int binary, const p3t_file_header_t *header, int n,
                            const p3t_bodies_t *bodies) {
    if (!path || !header || n < 0 || (n > 0 && (!bodies || !bodies->id || !bodies->mass || !bodies->pos ||
                                                !bodies->vel)))
        return P3T_IO_BAD_ARGUMENT;
    if (!binary && n > 0 && (!bodies->r_planet || !bodies->f)) return P3T_IO_BAD_ARGUMENT;
    FILE *fp = std::fopen(path, binary ? "wb" : "w");
    if (!fp) return P3T_IO_ERROR;
    p3t_file_header_t h = *header;
    h.n_body = n;
    int r = 0;
    const int nchunk = (n + CHUNK - 1) / CHUNK;
    if (binary) {
        FileHeaderRecord hr;
        std::memset(&hr, 0, sizeof hr);
        hr.n_body = h.n_body;
        hr.id_next = h.id_next;
        hr.time = h.time;
        std::memcpy(hr.e_init, h.e_init, sizeof hr.e_init);
        std::memcpy(hr.e_now, h.e_now, sizeof hr.e_now);
        r = write_all(fp, &hr, sizeof hr);
        std::vector<FPGravRecord> buf;
        for (int c = 0; c < nchunk && !r; c++) {
            const int lo = c * CHUNK, hi = std::min(n, lo + CHUNK);
            buf.resize((size_t)(hi - lo));
#pragma omp parallel for schedule(static)
            for (int i = lo; i < hi; i++) to_record(buf[(size_t)(i - lo)], bodies, i);
            r = write_all(fp, buf.data(), buf.size() * sizeof(FPGravRecord));
        }
    } else {
        std::string head;
        fmt_header(head, &h);
        r = write_all(fp, head.data(), head.size());
        // format a block of chunks in parallel, write it in order
        constexpr int BLOCK = 64;
        std::vector<std::string> text(BLOCK);
        for (int c0 = 0; c0 < nchunk && !r; c0 += BLOCK) {
            const int c1 = std::min(nchunk, c0 + BLOCK);
#pragma omp parallel for schedule(dynamic, 1)
            for (int c = c0; c < c1; c++) {
                std::string &s = text[(size_t)(c - c0)];
                s.clear();
                const int lo = c * CHUNK, hi = std::min(n, lo + CHUNK);
                s.reserve((size_t)(hi - lo) * 240);
                for (int i = lo; i < hi; i++) fmt_body(s, bodies, i);
            }
            for (int c = c0; c < c1 && !r; c++) r = write_all(fp, text[(size_t)(c - c0)].data(), text[(size_t)(c - c0)].size());
        }
    }
    if (std::fclose(fp) != 0 && !r) r = P3T_IO_ERROR;
    return r;
}

int p3t_collisions_write_host(const char *path, int append, int n, const p3t_collision_t *records) {
    if (!path || n < 0 || (n > 0 && !records)) return P3T_IO_BAD_ARGUMENT;
    FILE *fp = std::fopen(path, append ? "a" : "w");
    if (!fp) return P3T_IO_ERROR;
    int r = 0;
    char buf[1024];
    for (int k = 0; k < n && !r; k++) {
        const p3t_collision_t &c = records[k];
        // std::fixed, setprecision(8) for the time; std::scientific,
        // setprecision(15) for the doubles; tab-separated
        const int m = std::snprintf(
            buf, sizeof buf,
            "%.8f\t%lld\t%lld\t%d\t%lld\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t"
            "%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%.15e\t%d\t%.15e\t%.15e\n",
            c.time, c.id_imp, c.id_tar, c.n_frag, c.id_frag, c.mass_imp, c.mass_tar, c.mass_frag, c.pos_imp[0],
            c.pos_imp[1], c.pos_imp[2], c.pos_tar[0], c.pos_tar[1], c.pos_tar[2], c.vel_imp[0], c.vel_imp[1],
            c.vel_imp[2], c.vel_tar[0], c.vel_tar[1], c.vel_tar[2], c.flag, c.dpos_g_rel, c.dvel_g_rel);
        r = write_all(fp, buf, (size_t)m);
    }
    if (std::fclose(fp) != 0 && !r) r = P3T_IO_ERROR;
    return r;
}

int p3t_snapshot_read_host(const char *path, int binary, p3t_file_header_t *header, int cap,
                           const p3t_bodies_t *bodies) {
    if (!path || !header || cap < 0 || (cap > 0 && !bodies)) return P3T_IO_BAD_ARGUMENT;
    FILE *fp = std::fopen(path, binary ? "rb" : "r");
    if (!fp) return P3T_IO_ERROR;
    std::fseek(fp, 0, SEEK_END);
    const long size = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(fp);
        return P3T_IO_ERROR;
    }
    int n = 0;
    if (binary) {
        FileHeaderRecord hr;
        if (std::fread(&hr, sizeof hr, 1, fp) != 1) {
            std::fclose(fp);
            return P3T_IO_FORMAT;
        }
        std::memset(header, 0, sizeof *header);
        header->n_body = hr.n_body;
        header->id_next = hr.id_next;
        header->time = hr.time;
        std::memcpy(header->e_init, hr.e_init, sizeof hr.e_init);
        std::memcpy(header->e_now, hr.e_now, sizeof hr.e_now);
        n = hr.n_body;
        if (n < 0 || (long)(sizeof hr + (size_t)n * sizeof(FPGravRecord)) > size) {
            std::fclose(fp);
            return P3T_IO_FORMAT;
        }
        if (cap > 0) {
            if (n > cap) {
                std::fclose(fp);
                return P3T_IO_BAD_ARGUMENT;
            }
            std::vector<FPGravRecord> buf;
            for (int lo = 0; lo < n; lo += CHUNK) {
                const int hi = std::min(n, lo + CHUNK);
                buf.resize((size_t)(hi - lo));
                if (std::fread(buf.data(), sizeof(FPGravRecord), buf.size(), fp) != buf.size()) {
                    std::fclose(fp);
                    return P3T_IO_FORMAT;
                }
#pragma omp parallel for schedule(static)
                for (int i = lo; i < hi; i++) from_record(buf[(size_t)(i - lo)], bodies, i);
            }
        }
        std::fclose(fp);
        return n;
    }
    std::string text((size_t)size, '\0');
    const size_t got = std::fread(&text[0], 1, (size_t)size, fp);
    std::fclose(fp);
    text.resize(got);
    const char *p = text.data(), *end = p + text.size();
    // lines (skipping blank ones)
    std::vector<const char *> ls, le;
    for (const char *q = p; q < end;) {
        const char *e = line_end(q, end);
        if (!blank(q, e)) {
            ls.push_back(q);
            le.push_back(e);
        }
        q = e + 1;
    }
    // a header line has 13 fields, a body line 12
    size_t first = 0;
    std::memset(header, 0, sizeof *header);
    if (!ls.empty()) {
        int fields = 0;
        bool in = false;
        for (const char *q = ls[0]; q < le[0]; q++) {
            const bool sp = (*q == ' ' || *q == '\t' || *q == '\r');
            if (!sp && !in) fields++;
            in = !sp;
        }
        if (fields == 13) {
            if (!parse_header(ls[0], le[0], header)) return P3T_IO_FORMAT;
            first = 1;
        }
    }
    n = (int)(ls.size() - first);
    if (first && header->n_body != n) return P3T_IO_FORMAT;
    header->n_body = n;
    if (cap > 0) {
        if (n > cap) return P3T_IO_BAD_ARGUMENT;
        int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : bad)
        for (int i = 0; i < n; i++)
            if (!parse_body(ls[first + (size_t)i], le[first + (size_t)i], bodies, i)) bad++;
        if (bad) return P3T_IO_FORMAT;
    }
    return n;
}

}  // extern "C"
