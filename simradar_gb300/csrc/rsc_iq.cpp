/*
 * rsc_iq.cpp -- the .iq output file of simradar, written from a background
 * thread so that a pulse loop streaming I/Q blocks is not held by file I/O.
 *
 * Layout (the reader is matlab/simradariq.m; the writer simradar.c:340-366
 * with the headers of iq.h:20-41):
 *   file header, 1024 bytes:  RSParams (24 floats + uint32 range_count,
 *     rs_types.h:56-93), uint32 debris counts[8], char scan_mode[16],
 *     float scan_start, scan_end, scan_delta, uint32 simulation_seed, zero pad
 *   per pulse: 32-byte header (float time, el_deg, az_deg, zero pad), then
 *     range_count x float4 (Ih, Qh, Iv, Qv) with the gain applied
 * Little-endian, as the reference writes it on its x86-64 and arm64 hosts.
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rsc.h"

static_assert(sizeof(rsc_iq_params) == 100, "RSParams is 24 floats and a uint32");

namespace {

thread_local char g_iq_err[512] = "";

int iq_fail(int code, const char *msg) {
    snprintf(g_iq_err, sizeof(g_iq_err), "%s", msg);
    return code;
}

void put_u32(unsigned char *p, uint32_t v) {
    p[0] = (unsigned char)(v & 0xffu);
    p[1] = (unsigned char)((v >> 8) & 0xffu);
    p[2] = (unsigned char)((v >> 16) & 0xffu);
    p[3] = (unsigned char)((v >> 24) & 0xffu);
}

void put_f32(unsigned char *p, float f) {
    uint32_t v;
    memcpy(&v, &f, 4);
    put_u32(p, v);
}

}  // namespace

struct rsc_iq_writer {
    FILE *fid = nullptr;
    uint32_t range_count = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::vector<unsigned char>> queue;
    bool closing = false;
    bool writing = false;
    bool io_error = false;
    std::thread thread;

    void run() {
        for (;;) {
            std::vector<unsigned char> block;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv.wait(lock, [this] { return closing || !queue.empty(); });
                if (queue.empty()) return;
                block.swap(queue.front());
                queue.pop_front();
                writing = true;
            }
            const bool ok = fwrite(block.data(), 1, block.size(), fid) == block.size();
            {
                std::lock_guard<std::mutex> lock(mu);
                writing = false;
                if (!ok) io_error = true;
            }
            cv.notify_all();
        }
    }
};

extern "C" {

const char *rsc_iq_last_error(void) { return g_iq_err; }

int rsc_iq_open(const char *path, const rsc_iq_params *params, const uint32_t counts[RSC_MAX_TYPES],
                const char *scan_mode, float scan_start, float scan_end, float scan_delta, uint32_t seed,
                rsc_iq_writer **out) {
    if (path == nullptr || params == nullptr || out == nullptr) return iq_fail(RSC_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (params->range_count == 0 || params->range_count > RSC_MAX_GATES) {
        return iq_fail(RSC_ERR_ARG, "range_count outside [1, RSC_MAX_GATES]");
    }
    unsigned char hdr[1024];
    memset(hdr, 0, sizeof(hdr));
    float pf[24];
    memcpy(pf, params, sizeof(pf));
    for (int k = 0; k < 24; k++) put_f32(hdr + 4 * k, pf[k]);
    put_u32(hdr + 96, params->range_count);
    for (int k = 0; k < RSC_MAX_TYPES; k++) put_u32(hdr + 100 + 4 * k, counts ? counts[k] : 0u);
    if (scan_mode) {
        size_t n = strlen(scan_mode);
        memcpy(hdr + 132, scan_mode, n < 15 ? n : 15);
    }
    put_f32(hdr + 148, scan_start);
    put_f32(hdr + 152, scan_end);
    put_f32(hdr + 156, scan_delta);
    put_u32(hdr + 160, seed);
    FILE *fid = fopen(path, "wb");
    if (fid == nullptr) return iq_fail(RSC_ERR_ARG, "cannot create the I/Q file");
    if (fwrite(hdr, 1, sizeof(hdr), fid) != sizeof(hdr)) {
        fclose(fid);
        return iq_fail(RSC_ERR_ARG, "cannot write the I/Q file header");
    }
    rsc_iq_writer *w = new rsc_iq_writer();
    w->fid = fid;
    w->range_count = params->range_count;
    w->thread = std::thread([w] { w->run(); });
    *out = w;
    return RSC_OK;
}

int rsc_iq_write(rsc_iq_writer *w, uint32_t count, const float *times, const float *el_deg, const float *az_deg,
                 const float *pulses4, uint32_t row_gates, float gain) {
    if (w == nullptr || pulses4 == nullptr) return iq_fail(RSC_ERR_ARG, "NULL argument");
    if (row_gates < w->range_count) return iq_fail(RSC_ERR_ARG, "pulse rows shorter than range_count");
    const size_t per = 32 + (size_t)w->range_count * 16;
    std::vector<unsigned char> block(per * count, 0);
    for (uint32_t k = 0; k < count; k++) {
        unsigned char *p = block.data() + per * k;
        put_f32(p + 0, times ? times[k] : 0.0f);
        put_f32(p + 4, el_deg ? el_deg[k] : 0.0f);
        put_f32(p + 8, az_deg ? az_deg[k] : 0.0f);
        const float *src = pulses4 + (size_t)k * row_gates * 4;
        for (uint32_t g = 0; g < 4 * w->range_count; g++) put_f32(p + 32 + 4 * g, src[g] * gain);
    }
    std::lock_guard<std::mutex> lock(w->mu);
    if (w->io_error) return iq_fail(RSC_ERR_ARG, "an earlier write to the I/Q file failed");
    w->queue.push_back(std::move(block));
    w->cv.notify_all();
    return RSC_OK;
}

int rsc_iq_flush(rsc_iq_writer *w) {
    if (w == nullptr) return iq_fail(RSC_ERR_ARG, "NULL argument");
    std::unique_lock<std::mutex> lock(w->mu);
    w->cv.wait(lock, [w] { return w->queue.empty() && !w->writing; });
    if (w->io_error) return iq_fail(RSC_ERR_ARG, "a write to the I/Q file failed");
    fflush(w->fid);
    return RSC_OK;
}

int rsc_iq_close(rsc_iq_writer *w) {
    if (w == nullptr) return RSC_OK;
    {
        std::lock_guard<std::mutex> lock(w->mu);
        w->closing = true;
    }
    w->cv.notify_all();
    w->thread.join();
    const bool err = w->io_error;
    const int c = fclose(w->fid);
    delete w;
    if (err || c != 0) return iq_fail(RSC_ERR_ARG, "writing the I/Q file failed");
    return RSC_OK;
}

}  // extern "C"
