/*
 * rsc_les.cpp -- LES frames from the files of les.c, read ahead on a
 * background thread.
 *
 * Files (one LES folder, the folder les.c:71-126 finds):
 *   fort.10_2 (les.c:477-518): Fortran records; 16 bytes (the first record's
 *     length marker, nx, ny, nz as uint32), then three records of nx*ny*nz
 *     floats (x, y, z node coordinates), each after 8 bytes of markers.
 *   LES_mean_1_6_fnum<k>.dat, k = 1, 2, ... (les.c:212-244, les.c:350-386):
 *     a 4-byte marker, then per volume a float time stamp and the u, v, w, p,
 *     t planes (nx*ny*nz floats each), every field followed by 8 bytes.
 *     Volume n is in file n / 10 at volume n % 10 (LES_file_nblock, les.c:12).
 * Constants by configuration name: les.c:158-208 (v0 scales u, v, w; p0, t0
 * scale p and t; a, r the stretched-grid series; tp the period of a frame;
 * tr = 50, les.c:139).  Remap: les.c:388-406.
 *
 * Three frame buffers: the frame a caller holds, the one read ahead, and
 * one whose copy to the device may still be in flight.  A buffer that a copy
 * reads is refilled only after the copy's event completes.
 */
#include "rsc_les.h"

#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/stat.h>
#include <unistd.h>

#include <condition_variable>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int kEntries = 3;
constexpr uint32_t kFileVolumes = 10;   /* LES_file_nblock: volumes per file when indexing */
constexpr int kPlanes = 5;              /* u, v, w, p, t */

thread_local char g_les_err[512] = "";

int les_fail(int code, const char *msg) {
    snprintf(g_les_err, sizeof(g_les_err), "%s", msg);
    return code;
}

struct Entry {
    float *planes = nullptr;     /* kPlanes * nn floats, as stored in the file */
    float time = 0.0f;
    long long frame = -1;        /* -1: empty */
    bool reading = false;        /* being filled */
    int holds = 0;               /* callers holding the frame */
    bool pinned = false;         /* page-locked with cudaHostRegister */
    cudaEvent_t done = nullptr;  /* recorded after the last copy out of the buffer (made by release) */
    bool done_pending = false;
    unsigned long long stamp = 0;
};

}  // namespace

struct rsc_les_source {
    std::string dir, config;
    rsc_les_info info{};
    std::vector<std::string> files;
    std::vector<float> x, y, z;
    size_t nn = 0;
    Entry e[kEntries];
    std::mutex mu;
    std::condition_variable cv;
    long long want = -1;         /* frame for the thread to read next */
    bool closing = false;
    unsigned long long clock = 0;
    std::thread thread;
};

namespace {

bool read_exact(FILE *f, void *dst, size_t bytes) { return fread(dst, 1, bytes, f) == bytes; }

bool skip(FILE *f, long bytes) { return fseek(f, bytes, SEEK_CUR) == 0; }

int read_grid(rsc_les_source *s, const std::string &path) {
    FILE *f = fopen(path.c_str(), "rb");
    if (f == nullptr) return les_fail(RSC_ERR_ARG, "cannot open the LES grid file fort.10_2");
    uint32_t head[4];
    bool ok = read_exact(f, head, sizeof(head));
    const uint64_t count = ok ? (uint64_t)head[1] * head[2] * head[3] : 0;
    if (!ok || count == 0 || count >= (1ull << 31)) {
        fclose(f);
        return les_fail(RSC_ERR_ARG, "LES grid file: bad dimensions");
    }
    s->x.resize(count);
    s->y.resize(count);
    s->z.resize(count);
    ok = skip(f, 8) && read_exact(f, s->x.data(), count * 4) && skip(f, 8) && read_exact(f, s->y.data(), count * 4) &&
         skip(f, 8) && read_exact(f, s->z.data(), count * 4);
    fclose(f);
    if (!ok) return les_fail(RSC_ERR_ARG, "LES grid file shorter than its dimensions");
    s->info.nx = head[1];
    s->info.ny = head[2];
    s->info.nz = head[3];
    s->nn = (size_t)count;
    return RSC_OK;
}

void set_constants(rsc_les_source *s) {
    rsc_les_info &I = s->info;
    const char *c = s->config.c_str();
    I.tr = 50.0f;
    I.is_stretched = 0;
    if (!strcasecmp(c, "suctvort") || !strcasecmp(c, "suctvort_large")) {
        I.v0 = 100.0f;
        I.p0 = I.v0 * I.v0;
        I.t0 = I.v0 * I.v0;
        I.ax = I.ay = I.az = 2.0f;
        I.rx = I.ry = 1.0212f;
        I.rz = 1.05f;
        I.tp = 2.0f;
        I.is_stretched = 1;
    } else if (!strcasecmp(c, "twocell")) {
        I.v0 = 225.0f;
        I.p0 = I.v0 * I.v0;
        I.t0 = I.v0 * I.v0;
        I.ax = I.ay = I.az = 1.0f;
        I.rx = I.ry = I.rz = 1.0f;
        I.tp = 5.0f;
    } else if (!strcasecmp(c, "flat")) {
        const size_t nx = I.nx, nxy = (size_t)I.nx * I.ny;
        I.v0 = 100.0f;
        I.p0 = 1.0f;   /* p is used as cn2 */
        I.t0 = I.v0 * I.v0;
        I.ax = I.ay = I.az = 0.0f;
        I.rx = 1.0e3f * (s->x[nx > 1 ? 1 : 0] - s->x[0]);
        I.ry = 1.0e3f * (s->y[nx < s->nn ? nx : 0] - s->y[0]);
        I.rz = 1.0e3f * (s->z[nxy < s->nn ? nxy : 0] - s->z[0]);
        I.tp = 60.0f;
    } else {
        I.v0 = 100.0f;
        I.p0 = I.v0 * I.v0;
        I.t0 = I.v0 * I.v0;
        I.ax = I.ay = I.az = 1.0f;
        I.rx = I.ry = I.rz = 1.0f;
        I.tp = 5.0f;
    }
    /* the remap reads the config name case-sensitively (les.c:324) */
    I.p_for_cn2 = strcmp(c, "flat") == 0;
}

int find_files(rsc_les_source *s) {
    for (int k = 0;; k++) {
        std::string path = s->dir + "/LES_mean_1_6_fnum" + std::to_string(k + 1) + ".dat";
        if (access(path.c_str(), F_OK) != 0) break;
        if (s->files.empty()) {
            struct stat st;
            const uint64_t cells5 = (uint64_t)s->nn * kPlanes;
            if (stat(path.c_str(), &st) == 0) {
                s->info.volumes_per_file = (uint32_t)((uint64_t)st.st_size / (4 + 8 + cells5 * 4 + 8));
            } else {
                s->info.volumes_per_file = kFileVolumes;
            }
        }
        s->files.push_back(path);
    }
    if (s->files.empty()) return les_fail(RSC_ERR_ARG, "no LES_mean_1_6_fnum<k>.dat frame files in the LES folder");
    s->info.files = (uint32_t)s->files.size();
    s->info.frames = s->info.files * s->info.volumes_per_file;
    return RSC_OK;
}

/* Read frame `frame` into `planes` / `time` (no lock held). */
int read_frame(const rsc_les_source *s, uint32_t frame, float *planes, float *time, const char **why) {
    const size_t file_id = frame / kFileVolumes;
    if (file_id >= s->files.size()) {
        *why = "the frame's file does not exist";
        return RSC_ERR_ARG;
    }
    const long long per = (long long)(sizeof(float) + 8) + (long long)kPlanes * ((long long)s->nn * 4 + 8);
    const long long offset = 4 + (long long)(frame % kFileVolumes) * per;
    FILE *f = fopen(s->files[file_id].c_str(), "rb");
    if (f == nullptr) {
        *why = "cannot open the frame's file";
        return RSC_ERR_ARG;
    }
    bool ok = fseeko(f, (off_t)offset, SEEK_SET) == 0 && read_exact(f, time, sizeof(float)) && skip(f, 8);
    for (int p = 0; ok && p < kPlanes; p++) {
        ok = read_exact(f, planes + (size_t)p * s->nn, s->nn * sizeof(float)) && (p == kPlanes - 1 || skip(f, 8));
    }
    fclose(f);
    if (!ok) {
        *why = "the frame lies beyond the end of its file";
        return RSC_ERR_ARG;
    }
    return RSC_OK;
}

int find_entry(const rsc_les_source *s, long long frame) {
    for (int k = 0; k < kEntries; k++) {
        if (s->e[k].frame == frame) return k;
    }
    return -1;
}

/* least recently used buffer that nobody holds or fills, -1 if none */
int victim(const rsc_les_source *s) {
    int v = -1;
    for (int k = 0; k < kEntries; k++) {
        const Entry &E = s->e[k];
        if (E.holds || E.reading) continue;
        if (v < 0 || E.frame < 0 || (s->e[v].frame >= 0 && E.stamp < s->e[v].stamp)) v = k;
        if (E.frame < 0) break;
    }
    return v;
}

/* Fill entry k (claimed: reading set under the lock) with `frame`. */
int fill(rsc_les_source *s, int k, uint32_t frame, const char **why) {
    Entry &E = s->e[k];
    if (E.planes == nullptr) {
        void *p = nullptr;
        if (posix_memalign(&p, 4096, s->nn * kPlanes * sizeof(float)) != 0) {
            *why = "cannot allocate a frame buffer";
            return RSC_ERR_NOMEM;
        }
        E.planes = static_cast<float *>(p);
    }
    if (E.done_pending) {
        /* a copy out of this buffer may still run */
        cudaEventSynchronize(E.done);
        E.done_pending = false;
    }
    return read_frame(s, frame, E.planes, &E.time, why);
}

void claim(rsc_les_source *s, int k, uint32_t frame) {
    s->e[k].frame = frame;
    s->e[k].reading = true;
    s->e[k].stamp = ++s->clock;
}

void run(rsc_les_source *s) {
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        s->cv.wait(lock, [s] { return s->closing || s->want >= 0; });
        if (s->closing) return;
        const long long f = s->want;
        s->want = -1;
        if (find_entry(s, f) >= 0) continue;
        const int k = victim(s);
        if (k < 0) continue;   /* every buffer busy: the caller reads it itself */
        claim(s, k, (uint32_t)f);
        lock.unlock();
        const char *why = "";
        const int st = fill(s, k, (uint32_t)f, &why);
        lock.lock();
        s->e[k].reading = false;
        if (st) s->e[k].frame = -1;
        s->cv.notify_all();
    }
}

void request(rsc_les_source *s, uint32_t frame) {
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->want = frame;
    }
    s->cv.notify_all();
}

}  // namespace

namespace rscles {

const rsc_les_info &info(const rsc_les_source *src) { return src->info; }

int acquire(rsc_les_source *s, uint32_t frame, Held *out, const char **why) {
    if (frame >= s->info.frames) {
        *why = "frame outside the frames of the LES folder";
        return RSC_ERR_ARG;
    }
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        int k = find_entry(s, frame);
        if (k >= 0) {
            if (s->e[k].reading) {
                s->cv.wait(lock);
                continue;
            }
            Entry &E = s->e[k];
            E.holds++;
            E.stamp = ++s->clock;
            out->planes = E.planes;
            out->nn = s->nn;
            out->time = E.time;
            out->entry = k;
            break;
        }
        k = victim(s);
        if (k < 0) {
            s->cv.wait(lock);
            continue;
        }
        claim(s, k, frame);
        lock.unlock();
        const int st = fill(s, k, frame, why);
        lock.lock();
        s->e[k].reading = false;
        s->cv.notify_all();
        if (st) {
            s->e[k].frame = -1;
            return st;
        }
    }
    lock.unlock();
    /* what to read next (les.c:680-681) */
    request(s, frame + 1 == s->info.frames ? 0u : frame + 1);
    return RSC_OK;
}

int pin(rsc_les_source *s, const Held &h, const char **why) {
    std::lock_guard<std::mutex> lock(s->mu);   /* callers holding the same buffer */
    Entry &E = s->e[h.entry];
    if (E.pinned) return RSC_OK;
    cudaError_t e = cudaHostRegister(E.planes, s->nn * kPlanes * sizeof(float), cudaHostRegisterPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *why = cudaGetErrorString(e);
        return RSC_ERR_CUDA;
    }
    E.pinned = true;
    return RSC_OK;
}

void release(rsc_les_source *s, const Held &h, cudaStream_t copy_stream) {
    std::lock_guard<std::mutex> lock(s->mu);
    Entry &E = s->e[h.entry];
    if (copy_stream != nullptr) {
        cudaError_t e = cudaSuccess;
        if (E.done == nullptr) e = cudaEventCreateWithFlags(&E.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(E.done, copy_stream);
        if (e == cudaSuccess) {
            E.done_pending = true;
        } else {
            cudaGetLastError();
            cudaStreamSynchronize(copy_stream);   /* no event: wait for the copy here */
        }
    }
    E.holds--;
    s->cv.notify_all();
}

}  // namespace rscles

extern "C" {

const char *rsc_les_last_error(void) { return g_les_err; }

int rsc_les_open(const char *dir, const char *config, rsc_les_source **out) {
    if (dir == nullptr || config == nullptr || out == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    *out = nullptr;
    rsc_les_source *s = new rsc_les_source();
    s->dir = dir;
    s->config = config;
    int st = read_grid(s, s->dir + "/fort.10_2");
    if (st == RSC_OK) set_constants(s);
    if (st == RSC_OK) st = find_files(s);
    if (st) {
        delete s;
        return st;
    }
    s->thread = std::thread(run, s);
    request(s, 0);   /* LES_init waits for the first frame (les.c:275-279) */
    *out = s;
    return RSC_OK;
}

int rsc_les_get_info(rsc_les_source *src, rsc_les_info *info) {
    if (src == nullptr || info == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    *info = src->info;
    return RSC_OK;
}

int rsc_les_grid(rsc_les_source *src, float *x, float *y, float *z) {
    if (src == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    if (x) memcpy(x, src->x.data(), src->nn * sizeof(float));
    if (y) memcpy(y, src->y.data(), src->nn * sizeof(float));
    if (z) memcpy(z, src->z.data(), src->nn * sizeof(float));
    return RSC_OK;
}

int rsc_les_descriptor(const rsc_les_info *I, float desc[16]) {
    if (I == nullptr || desc == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    for (int k = 0; k < 16; k++) desc[k] = 0.0f;
    uint32_t spacing = 0;
    if (I->is_stretched) {
        /* rs.c:3057-3059: k = log1p((r - 1) / a * |p|) / log(r) + (n - 1) / 2 */
        spacing = 7u;
        desc[0] = (float)(1.0 / log((double)I->rx));
        desc[4] = (I->rx - 1.0f) / I->ax;
        desc[8] = 0.5f * (float)(I->nx - 1);
        desc[1] = (float)(1.0 / log((double)I->ry));
        desc[5] = (I->ry - 1.0f) / I->ay;
        desc[9] = 0.5f * (float)(I->ny - 1);
        desc[2] = (float)(1.0 / log((double)I->rz));
        desc[6] = (I->rz - 1.0f) / I->az;
        desc[10] = 0.0f;
    } else {
        /* rs.c:3076-3078: index = pos / spacing + centre */
        desc[0] = 1.0f / I->rx;
        desc[4] = (float)(I->nx - 1) * 0.5f;
        desc[8] = (float)I->nx - 1.0f;
        desc[1] = 1.0f / I->ry;
        desc[5] = (float)(I->ny - 1) * 0.5f;
        desc[9] = (float)I->ny - 1.0f;
        desc[2] = 1.0f / I->rz;
        desc[6] = 0.0f;
        desc[10] = (float)I->nz - 1.0f;
    }
    memcpy(&desc[7], &spacing, sizeof(float));   /* the spacing bits as a float (rs.c:2945) */
    desc[3] = I->tr;
    return RSC_OK;
}

int rsc_les_read(rsc_les_source *src, uint32_t frame, float *uvwt4, float *cpxx4, float *time) {
    if (src == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    rscles::Held h;
    const char *why = "";
    int st = rscles::acquire(src, frame, &h, &why);
    if (st) return les_fail(st, why);
    const rsc_les_info &I = src->info;
    const size_t nn = h.nn;
    const float *u = h.planes, *v = u + nn, *w = v + nn, *p = w + nn, *t = p + nn;
    for (size_t k = 0; k < nn; k++) {
        if (uvwt4) {
            uvwt4[4 * k + 0] = u[k] * I.v0;
            uvwt4[4 * k + 1] = v[k] * I.v0;
            uvwt4[4 * k + 2] = w[k] * I.v0;
            uvwt4[4 * k + 3] = t[k] * I.t0;
        }
        if (cpxx4) {
            const float pp = p[k] * I.p0;
            cpxx4[4 * k + 0] = I.p_for_cn2 ? pp : 0.0f;
            cpxx4[4 * k + 1] = I.p_for_cn2 ? 0.0f : pp;
            cpxx4[4 * k + 2] = 0.0f;
            cpxx4[4 * k + 3] = 0.0f;
        }
    }
    if (time) *time = h.time;
    rscles::release(src, h, nullptr);
    return RSC_OK;
}

int rsc_les_prefetch(rsc_les_source *src, uint32_t frame) {
    if (src == nullptr) return les_fail(RSC_ERR_ARG, "NULL argument");
    if (frame >= src->info.frames) return les_fail(RSC_ERR_ARG, "frame outside the frames of the LES folder");
    request(src, frame);
    return RSC_OK;
}

int rsc_les_close(rsc_les_source *src) {
    if (src == nullptr) return RSC_OK;
    {
        std::lock_guard<std::mutex> lock(src->mu);
        src->closing = true;
    }
    src->cv.notify_all();
    src->thread.join();
    for (Entry &E : src->e) {
        if (E.done_pending) cudaEventSynchronize(E.done);
        if (E.done) cudaEventDestroy(E.done);
        if (E.pinned) cudaHostUnregister(E.planes);
        free(E.planes);
    }
    delete src;
    return RSC_OK;
}

}  // extern "C"
