// Snapshot and sanity-record output in NetCDF (classic encoding), the C ABI of the
// "Snapshot output" and "Sanity-check records" sections of include/swe_gb300.h.
//
// Device snapshots: the reference stops the solver at every save_every step, copies
// the whole ghosted state to the host, packs the interior on the CPU and writes it
// (cuda_solver.hpp:211-219, netCDF_writer.cpp:73-83,135-149).  Here a kernel on the
// context's stream packs U^n's interior straight into the file's byte order (x slow,
// y contiguous, big-endian) in a device staging buffer; the context's next steps queue
// behind that kernel only.  A writer thread then moves the staging buffer to disk in
// chunks: device-to-host copies into a ring of pinned buffers on its own stream, each
// written to the file as soon as its copy lands, so that copies, file writes and the
// solver's kernels overlap.  Two staging buffers let a second snapshot be packed while
// the first is still being written.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/swe_gb300.h"
#include "swe_ctx.h"
#include "swe_ncfile.h"

using swe::nc::ClassicFile;

namespace {

constexpr int kRing = 4;                       // pinned chunk buffers
constexpr size_t kChunk = size_t(64) << 20;    // bytes per device-to-host chunk
constexpr size_t kHeaderReserve = 8192;        // room for the late run metadata

__device__ __forceinline__ unsigned long long bswap64(unsigned long long v) {
    const unsigned lo = (unsigned)v, hi = (unsigned)(v >> 32);
    return ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | __byte_perm(hi, 0, 0x0123);
}

// Interior of (h, hu, hv) -> out[f][i][j], big-endian doubles.  One row per block
// iteration; the threads of a block sweep j, so reads and writes are coalesced.
__global__ void k_pack_be_f64(const double *__restrict__ h, const double *__restrict__ hu,
                              const double *__restrict__ hv, int Nx, int Ny, long long P,
                              unsigned long long *__restrict__ out) {
    const long long plane = (long long)Nx * Ny;
    for (int i = blockIdx.x; i < Nx; i += gridDim.x) {
        const long long src = (long long)(i + 2) * P + 2, dst = (long long)i * Ny;
        for (int j = threadIdx.x; j < Ny; j += blockDim.x) {
            out[dst + j] = bswap64(__double_as_longlong(h[src + j]));
            out[plane + dst + j] = bswap64(__double_as_longlong(hu[src + j]));
            out[2 * plane + dst + j] = bswap64(__double_as_longlong(hv[src + j]));
        }
    }
}

// FP32-mixed state (eta, hu, hv over FP32 B): h = eta - B in FP64 (exact), hu and hv
// widened, the conversion swe_download applies.
__global__ void k_pack_be_f32(const float *__restrict__ e, const float *__restrict__ hu,
                              const float *__restrict__ hv, const float *__restrict__ B,
                              int Nx, int Ny, long long P, unsigned long long *__restrict__ out) {
    const long long plane = (long long)Nx * Ny;
    for (int i = blockIdx.x; i < Nx; i += gridDim.x) {
        const long long src = (long long)(i + 2) * P + 2, dst = (long long)i * Ny;
        for (int j = threadIdx.x; j < Ny; j += blockDim.x) {
            const double hh = (double)e[src + j] - (double)B[src + j];
            out[dst + j] = bswap64(__double_as_longlong(hh));
            out[plane + dst + j] = bswap64(__double_as_longlong((double)hu[src + j]));
            out[2 * plane + dst + j] = bswap64(__double_as_longlong((double)hv[src + j]));
        }
    }
}

bool nonempty(const char *s) { return s && s[0]; }

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct swe_snapshot {
    ClassicFile f;
    int Nx = 0, Ny = 0;
    int v_time = -1, v_x = -1, v_y = -1, v_h = -1, v_hu = -1, v_hv = -1, v_B = -1;
    bool metadata_written = false, bathymetry_written = false, closed = false;
    long long next_record = 0;  // records issued (written or queued)
    std::string err;            // caller-side message

    // Device pipeline, set up by the first device write.
    int device = -1;
    cudaStream_t copy = nullptr;
    void *staging[2]{};
    cudaEvent_t packed[2]{};
    unsigned char *ring = nullptr;  // kRing pinned chunks
    size_t chunk = 0;               // bytes per chunk: min(kChunk, one record's fields)
    cudaEvent_t landed[kRing]{};
    int next_slot = 0;

    struct Job {
        int slot;
        long long rec;
        double time;
    };
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Job> jobs;  // the front job stays queued until it is on disk
    bool busy[2]{};
    bool stop = false;
    int status = SWE_OK;
    std::string werr;
    double copy_s = 0.0, write_s = 0.0;
    long long bytes = 0;
};

namespace {

int snap_fail(swe_snapshot *s, int status, const std::string &m) {
    if (s) s->err = m;
    return status;
}

size_t plane_bytes(const swe_snapshot *s) { return (size_t)s->Nx * (size_t)s->Ny * sizeof(double); }

// Packs rows [i0, i1) of a ghosted host array's interior into be (big-endian).
void pack_rows_host(const double *A, int Ny, int i0, int i1, unsigned char *be) {
    const size_t row = (size_t)Ny + 4;
    for (int i = i0; i < i1; ++i)
        swe::nc::store_be64(be + (size_t)(i - i0) * Ny * 8, A + (size_t)(i + 2) * row + 2, Ny);
}

// Writes the interior of a ghosted host array into a fixed variable or a record slab,
// through a bounded bounce buffer.
bool write_host_field(swe_snapshot *s, int var, long long rec, const double *A) {
    const int rows_per = (int)std::max<size_t>(1, kChunk / ((size_t)s->Ny * 8));
    std::vector<unsigned char> buf((size_t)std::min(rows_per, s->Nx) * s->Ny * 8);
    for (int i0 = 0; i0 < s->Nx; i0 += rows_per) {
        const int i1 = std::min(s->Nx, i0 + rows_per);
        pack_rows_host(A, s->Ny, i0, i1, buf.data());
        const size_t n = (size_t)(i1 - i0) * s->Ny * 8;
        const uint64_t off = (uint64_t)i0 * s->Ny * 8;
        const bool ok = rec < 0 ? s->f.write_fixed(var, buf.data(), n, off)
                                : s->f.write_record(var, (uint64_t)rec, buf.data(), n, off);
        if (!ok) return false;
    }
    return true;
}

// Moves one packed staging buffer to record job.rec.  Runs on the writer thread.
int run_job(swe_snapshot *s, const swe_snapshot::Job &job, std::string &msg, double &copy_s,
            double &write_s, long long &bytes) {
    const size_t pb = plane_bytes(s);
    const size_t total = 3 * pb;
    const size_t chunk = s->chunk;
    const size_t nchunks = (total + chunk - 1) / chunk;
    const int vars[3] = {s->v_h, s->v_hu, s->v_hv};
    const unsigned char *src = static_cast<const unsigned char *>(s->staging[job.slot]);
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        msg = std::string("snapshot: ") + what + " failed: " + cudaGetErrorString(e);
        return SWE_ERR_CUDA;
    };
    cudaError_t e = cudaStreamWaitEvent(s->copy, s->packed[job.slot], 0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
    auto issue = [&](size_t c) {
        const size_t off = c * chunk, n = std::min(chunk, total - off);
        unsigned char *dst = s->ring + (c % kRing) * chunk;
        cudaError_t r = cudaMemcpyAsync(dst, src + off, n, cudaMemcpyDeviceToHost, s->copy);
        if (r == cudaSuccess) r = cudaEventRecord(s->landed[c % kRing], s->copy);
        return r;
    };
    for (size_t c = 0; c < nchunks && c < (size_t)kRing; ++c)
        if ((e = issue(c)) != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
    for (size_t c = 0; c < nchunks; ++c) {
        auto t0 = std::chrono::steady_clock::now();
        if ((e = cudaEventSynchronize(s->landed[c % kRing])) != cudaSuccess)
            return cuda_fail(e, "cudaEventSynchronize");
        copy_s += seconds_since(t0);
        t0 = std::chrono::steady_clock::now();
        // A chunk may span the h / hu / hv boundary: split it per variable.
        size_t off = c * chunk;
        const size_t end = std::min(total, off + chunk);
        const unsigned char *p = s->ring + (c % kRing) * chunk;
        while (off < end) {
            const size_t f = off / pb, in = off - f * pb;
            const size_t n = std::min(end - off, pb - in);
            if (!s->f.write_record(vars[f], (uint64_t)job.rec, p, n, in)) {
                msg = "snapshot: " + s->f.error();
                return SWE_ERR_IO;
            }
            p += n;
            off += n;
        }
        write_s += seconds_since(t0);
        bytes += (long long)(end - c * chunk);
        if (c + kRing < nchunks && (e = issue(c + kRing)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpyAsync");
    }
    unsigned char tb[8];
    swe::nc::store_be64(tb, &job.time, 1);
    if (!s->f.write_record(s->v_time, (uint64_t)job.rec, tb, 8) ||
        !s->f.set_numrecs((uint64_t)job.rec + 1)) {
        msg = "snapshot: " + s->f.error();
        return SWE_ERR_IO;
    }
    return SWE_OK;
}

void worker_main(swe_snapshot *s) {
    cudaSetDevice(s->device);
    for (;;) {
        swe_snapshot::Job job;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return s->stop || !s->jobs.empty(); });
            if (s->jobs.empty()) return;
            job = s->jobs.front();
        }
        std::string msg;
        const bool skip = [&] {
            std::lock_guard<std::mutex> lk(s->mu);
            return s->status != SWE_OK;
        }();
        double cs = 0.0, ws = 0.0;
        long long by = 0;
        const int st = skip ? SWE_OK : run_job(s, job, msg, cs, ws, by);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->copy_s += cs;
            s->write_s += ws;
            s->bytes += by;
            if (st != SWE_OK && s->status == SWE_OK) {
                s->status = st;
                s->werr = msg;
            }
            s->busy[job.slot] = false;
            s->jobs.pop_front();
        }
        s->cv.notify_all();
    }
}

// Stream-ordered device resources, created on ctx's device at the first device write.
int setup_device(swe_snapshot *s, swe_ctx *c) {
    if (s->device >= 0) {
        if (s->device != c->p.device)
            return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write: context on another device");
        return SWE_OK;
    }
    cudaError_t e = cudaSetDevice(c->p.device);
    const size_t total = 3 * plane_bytes(s);
    s->chunk = std::min(kChunk, total);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaMalloc(&s->staging[k], total);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->packed[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&s->ring, kRing * s->chunk, cudaHostAllocDefault);
    for (int k = 0; k < kRing && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&s->landed[k], cudaEventDisableTiming | cudaEventBlockingSync);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return snap_fail(s, e == cudaErrorMemoryAllocation ? SWE_ERR_BAD_ARG : SWE_ERR_CUDA,
                         std::string("swe_snapshot_write: device setup failed: ") +
                             cudaGetErrorString(e));
    }
    s->device = c->p.device;
    s->worker = std::thread(worker_main, s);
    return SWE_OK;
}

void release_device(swe_snapshot *s) {
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv.notify_all();
        s->worker.join();
    }
    if (s->device < 0) return;
    cudaSetDevice(s->device);
    if (s->copy) cudaStreamSynchronize(s->copy);
    for (int k = 0; k < 2; ++k) {
        if (s->staging[k]) cudaFree(s->staging[k]);
        if (s->packed[k]) cudaEventDestroy(s->packed[k]);
        s->staging[k] = nullptr;
        s->packed[k] = nullptr;
    }
    for (int k = 0; k < kRing; ++k) {
        if (s->landed[k]) cudaEventDestroy(s->landed[k]);
        s->landed[k] = nullptr;
    }
    if (s->ring) cudaFreeHost(s->ring);
    if (s->copy) cudaStreamDestroy(s->copy);
    s->ring = nullptr;
    s->copy = nullptr;
    cudaGetLastError();
    s->device = -1;
}

// Waits for every queued device record; returns the writer's first error.
int drain(swe_snapshot *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.wait(lk, [&] { return s->jobs.empty(); });
    if (s->status != SWE_OK) s->err = s->werr;
    return s->status;
}

}  // namespace

extern "C" {

int swe_snapshot_open(const char *path, const swe_snapshot_params *p, swe_snapshot **out) try {
    if (!out) return SWE_ERR_BAD_ARG;
    *out = nullptr;
    if (!path || !p || p->Nx < 1 || p->Ny < 1 || !(p->dx > 0.0) || !(p->dy > 0.0) ||
        (p->format != 0 && p->format != 2 && p->format != 5))
        return SWE_ERR_BAD_ARG;
    swe_snapshot *s = new (std::nothrow) swe_snapshot();
    if (!s) return SWE_ERR_BAD_ARG;
    s->Nx = p->Nx;
    s->Ny = p->Ny;
    const uint64_t field = (uint64_t)p->Nx * (uint64_t)p->Ny * 8;
    const bool fits2 = field <= ClassicFile::kCdf2VarLimit && p->Nx <= 0x7fffffff;
    if (p->format == 2 && !fits2) {
        delete s;
        return SWE_ERR_BAD_ARG;  // a field of 4 GiB or more needs CDF-5
    }
    const int version = p->format == 0 ? (fits2 ? 2 : 5) : p->format;
    ClassicFile &f = s->f;
    bool ok = f.create(path, version);
    // define_file_structure (netCDF_writer.cpp:29-56): same names, order and types.
    int d_time = -1, d_x = -1, d_y = -1;
    if (ok) {
        d_time = f.add_dim("time", 0);
        d_x = f.add_dim("x", (uint64_t)p->Nx);
        d_y = f.add_dim("y", (uint64_t)p->Ny);
        s->v_time = f.add_var("time", swe::nc::NC_DOUBLE, {d_time});
        s->v_x = f.add_var("x", swe::nc::NC_DOUBLE, {d_x});
        s->v_y = f.add_var("y", swe::nc::NC_DOUBLE, {d_y});
        s->v_h = f.add_var("h", swe::nc::NC_DOUBLE, {d_time, d_x, d_y});
        s->v_hu = f.add_var("hu", swe::nc::NC_DOUBLE, {d_time, d_x, d_y});
        s->v_hv = f.add_var("hv", swe::nc::NC_DOUBLE, {d_time, d_x, d_y});
        s->v_B = f.add_var("B", swe::nc::NC_DOUBLE, {d_x, d_y});
        ok = s->v_B >= 0;
    }
    if (ok && nonempty(p->unit_x)) ok = f.put_att_text(s->v_x, "units", p->unit_x);
    if (ok && nonempty(p->unit_y)) ok = f.put_att_text(s->v_y, "units", p->unit_y);
    if (ok && nonempty(p->unit_h))
        ok = f.put_att_text(s->v_h, "units", p->unit_h) && f.put_att_text(s->v_B, "units", p->unit_h);
    if (ok && nonempty(p->unit_time)) ok = f.put_att_text(s->v_time, "units", p->unit_time);
    if (ok) ok = f.put_att_int(-1, "save_every", p->save_every);
    if (ok) ok = f.enddef(kHeaderReserve);
    if (ok) {
        // write_coordinates (:58-71): x_center(i) = (i + 0.5) * dx (grid.hpp:22-23)
        std::vector<double> x((size_t)p->Nx), y((size_t)p->Ny);
        for (int i = 0; i < p->Nx; ++i) x[(size_t)i] = (i + 0.5) * p->dx;
        for (int j = 0; j < p->Ny; ++j) y[(size_t)j] = (j + 0.5) * p->dy;
        swe::nc::store_be64(x.data(), x.data(), x.size());
        swe::nc::store_be64(y.data(), y.data(), y.size());
        ok = f.write_fixed(s->v_x, x.data(), x.size() * 8) &&
             f.write_fixed(s->v_y, y.data(), y.size() * 8);
    }
    if (!ok) {
        delete s;
        return SWE_ERR_IO;
    }
    *out = s;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_snapshot_bathymetry(swe_snapshot *s, const double *B) try {
    if (!s || !B) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_bathymetry: null argument");
    if (s->closed) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_bathymetry: file closed");
    if (s->bathymetry_written) return SWE_OK;  // netCDF_writer.cpp:87-89
    if (!write_host_field(s, s->v_B, -1, B)) return snap_fail(s, SWE_ERR_IO, s->f.error());
    s->bathymetry_written = true;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_snapshot_metadata(swe_snapshot *s, double dt, const char *backend,
                          const char *riemann_solver, const char *reconstruction,
                          const char *time_integrator, const char *boundary_condition,
                          const char *bathymetry) try {
    if (!s) return SWE_ERR_BAD_ARG;
    if (s->closed) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_metadata: file closed");
    // netCDF_writer.cpp:107-133: backend alone does not trigger the metadata.
    if (s->metadata_written ||
        !(!std::isnan(dt) || nonempty(riemann_solver) || nonempty(reconstruction) ||
          nonempty(time_integrator) || nonempty(boundary_condition) || nonempty(bathymetry)))
        return SWE_OK;
    ClassicFile &f = s->f;
    bool ok = true;
    if (!std::isnan(dt)) ok = f.put_att_double(-1, "dt", dt);
    const char *names[6] = {"backend", "riemann_solver", "reconstruction",
                            "time_integrator", "boundary_condition", "bathymetry"};
    const char *vals[6] = {backend, riemann_solver, reconstruction,
                           time_integrator, boundary_condition, bathymetry};
    for (int k = 0; k < 6 && ok; ++k)
        if (nonempty(vals[k])) ok = f.put_att_text(-1, names[k], vals[k]);
    if (!ok) return snap_fail(s, SWE_ERR_IO, f.error());
    s->metadata_written = true;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_snapshot_write_host(swe_snapshot *s, double time, const double *h, const double *hu,
                            const double *hv) try {
    if (!s || !h || !hu || !hv)
        return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write_host: null argument");
    if (s->closed) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write_host: file closed");
    if (s->device >= 0) {
        const int st = drain(s);
        if (st) return st;
    }
    const long long rec = s->next_record;
    unsigned char tb[8];
    swe::nc::store_be64(tb, &time, 1);
    // write_snapshot (:135-149): time, then h, hu, hv of record next_record_.
    if (!s->f.write_record(s->v_time, (uint64_t)rec, tb, 8) ||
        !write_host_field(s, s->v_h, rec, h) || !write_host_field(s, s->v_hu, rec, hu) ||
        !write_host_field(s, s->v_hv, rec, hv) || !s->f.set_numrecs((uint64_t)rec + 1))
        return snap_fail(s, SWE_ERR_IO, s->f.error());
    s->next_record = rec + 1;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_snapshot_write(swe_snapshot *s, swe_ctx *c, double time) try {
    if (!s || !c) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write: null argument");
    if (s->closed) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write: file closed");
    if (!c->uploaded) return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write: no state uploaded");
    if (c->p.Nx != s->Nx || c->p.Ny != s->Ny)
        return snap_fail(s, SWE_ERR_BAD_ARG, "swe_snapshot_write: grid size differs from the file's");
    int st = setup_device(s, c);
    if (st) return st;
    const int slot = s->next_slot;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv.wait(lk, [&] { return !s->busy[slot] || s->status != SWE_OK; });
        if (s->status != SWE_OK) {
            s->err = s->werr;
            return s->status;
        }
    }
    cudaError_t e = cudaSetDevice(c->p.device);
    const int blocks = std::min(s->Nx, 8 * c->num_sms);
    if (e == cudaSuccess) {
        if (c->p.precision == SWE_PRECISION_FP32_MIXED)
            k_pack_be_f32<<<blocks, 256, 0, c->stream>>>(
                static_cast<const float *>(c->Un[0]), static_cast<const float *>(c->Un[1]),
                static_cast<const float *>(c->Un[2]), static_cast<const float *>(c->B), s->Nx,
                s->Ny, c->pitch, static_cast<unsigned long long *>(s->staging[slot]));
        else
            k_pack_be_f64<<<blocks, 256, 0, c->stream>>>(
                static_cast<const double *>(c->Un[0]), static_cast<const double *>(c->Un[1]),
                static_cast<const double *>(c->Un[2]), s->Nx, s->Ny, c->pitch,
                static_cast<unsigned long long *>(s->staging[slot]));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(s->packed[slot], c->stream);
    if (e != cudaSuccess)
        return snap_fail(s, SWE_ERR_CUDA,
                         std::string("swe_snapshot_write: pack failed: ") + cudaGetErrorString(e));
    ++c->launches;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->busy[slot] = true;
        s->jobs.push_back({slot, s->next_record, time});
    }
    s->cv.notify_all();
    ++s->next_record;
    s->next_slot ^= 1;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_CUDA;
}

int swe_snapshot_flush(swe_snapshot *s) {
    if (!s) return SWE_ERR_BAD_ARG;
    if (s->device < 0) return SWE_OK;
    return drain(s);
}

long long swe_snapshot_records(const swe_snapshot *s) { return s ? s->next_record : 0; }

int swe_snapshot_stats(const swe_snapshot *s, double *copy_s, double *write_s, long long *bytes) {
    if (!s || !copy_s || !write_s || !bytes) return SWE_ERR_BAD_ARG;
    swe_snapshot *m = const_cast<swe_snapshot *>(s);
    std::lock_guard<std::mutex> lk(m->mu);
    *copy_s = s->copy_s;
    *write_s = s->write_s;
    *bytes = s->bytes;
    return SWE_OK;
}

int swe_snapshot_close(swe_snapshot *s) try {
    if (!s) return SWE_ERR_BAD_ARG;
    if (s->closed) return SWE_OK;
    int st = s->device >= 0 ? drain(s) : SWE_OK;
    release_device(s);
    if (st == SWE_OK && !s->bathymetry_written) {
        // An unwritten B reads as netCDF's default fill value, as in the reference's file.
        std::vector<double> fill((size_t)s->Ny, swe::nc::kFillDouble);
        swe::nc::store_be64(fill.data(), fill.data(), fill.size());
        for (int i = 0; i < s->Nx && st == SWE_OK; ++i)
            if (!s->f.write_fixed(s->v_B, fill.data(), fill.size() * 8, (uint64_t)i * s->Ny * 8))
                st = snap_fail(s, SWE_ERR_IO, s->f.error());
    }
    if (!s->f.close() && st == SWE_OK) st = snap_fail(s, SWE_ERR_IO, s->f.error());
    s->closed = true;
    return st;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

void swe_snapshot_destroy(swe_snapshot *s) try {
    if (!s) return;
    swe_snapshot_close(s);
    delete s;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
}

const char *swe_snapshot_last_error(const swe_snapshot *s) {
    return s ? s->err.c_str() : "null snapshot";
}

}  // extern "C"

// ---- Sanity-check records ----------------------------------------------------------------

struct swe_sanity_log {
    ClassicFile f;
    int v_step = -1, v_time = -1, v_err = -1, v_hmin = -1;
    unsigned long long next_record = 0;
    bool closed = false;
    std::string err;
};

extern "C" {

int swe_sanity_log_open(const char *path, const char *time_unit, const char *h_unit,
                        int save_every, double dt, const char *backend,
                        const char *riemann_solver, const char *reconstruction,
                        const char *time_integrator, const char *boundary_condition,
                        const char *bathymetry, swe_sanity_log **out) try {
    if (!out) return SWE_ERR_BAD_ARG;
    *out = nullptr;
    if (!path) return SWE_ERR_BAD_ARG;
    swe_sanity_log *l = new (std::nothrow) swe_sanity_log();
    if (!l) return SWE_ERR_BAD_ARG;
    ClassicFile &f = l->f;
    auto str = [](const char *s) { return std::string(s ? s : ""); };
    // define_file_structure (sanity_checks_netcdf_writer.cpp:25-59)
    bool ok = f.create(path, 5);
    if (ok) {
        const int d = f.add_dim("record", 0);
        l->v_step = f.add_var("step", swe::nc::NC_UINT64, {d});
        l->v_time = f.add_var("time", swe::nc::NC_DOUBLE, {d});
        l->v_err = f.add_var("mass_rel_err", swe::nc::NC_DOUBLE, {d});
        l->v_hmin = f.add_var("h_min", swe::nc::NC_DOUBLE, {d});
        ok = l->v_hmin >= 0 && f.put_att_text(l->v_step, "long_name", "time_step_index") &&
             f.put_att_text(l->v_time, "long_name", "physical_time");
    }
    if (ok && nonempty(time_unit)) ok = f.put_att_text(l->v_time, "units", time_unit);
    if (ok)
        ok = f.put_att_text(l->v_err, "long_name", "relative_mass_error") &&
             f.put_att_text(l->v_err, "units", "1") &&
             f.put_att_text(l->v_hmin, "long_name", "minimum_water_height");
    if (ok && nonempty(h_unit)) ok = f.put_att_text(l->v_hmin, "units", h_unit);
    // The reference stores these strings even when empty (zero-length text attributes).
    if (ok)
        ok = f.put_att_int(-1, "save_every", save_every) && f.put_att_double(-1, "dt", dt) &&
             f.put_att_text(-1, "backend", str(backend)) &&
             f.put_att_text(-1, "riemann_solver", str(riemann_solver)) &&
             f.put_att_text(-1, "reconstruction", str(reconstruction)) &&
             f.put_att_text(-1, "time_integrator", str(time_integrator)) &&
             f.put_att_text(-1, "boundary_condition", str(boundary_condition)) &&
             f.put_att_text(-1, "bathymetry", str(bathymetry)) &&
             f.put_att_int(-1, "mass_conservation_enabled", 1) &&
             f.put_att_int(-1, "positivity_enabled", 1) && f.enddef(0);
    if (!ok) {
        delete l;
        return SWE_ERR_IO;
    }
    *out = l;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_sanity_log_write(swe_sanity_log *l, unsigned long long step, double time,
                         double rel_err, double h_min) try {
    if (!l) return SWE_ERR_BAD_ARG;
    if (l->closed) {
        l->err = "swe_sanity_log_write: file closed";
        return SWE_ERR_BAD_ARG;
    }
    const uint64_t r = l->next_record;
    unsigned char b[8];
    uint64_t sv = step;
    bool ok = true;
    swe::nc::store_be64(b, &sv, 1);
    ok = ok && l->f.write_record(l->v_step, r, b, 8);
    swe::nc::store_be64(b, &time, 1);
    ok = ok && l->f.write_record(l->v_time, r, b, 8);
    swe::nc::store_be64(b, &rel_err, 1);
    ok = ok && l->f.write_record(l->v_err, r, b, 8);
    swe::nc::store_be64(b, &h_min, 1);
    ok = ok && l->f.write_record(l->v_hmin, r, b, 8) && l->f.set_numrecs(r + 1);
    if (!ok) {
        l->err = l->f.error();
        return SWE_ERR_IO;
    }
    l->next_record = r + 1;
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

int swe_sanity_log_close(swe_sanity_log *l) try {
    if (!l) return SWE_ERR_BAD_ARG;
    if (l->closed) return SWE_OK;
    l->closed = true;
    if (!l->f.close()) {
        l->err = l->f.error();
        return SWE_ERR_IO;
    }
    return SWE_OK;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
    return SWE_ERR_IO;
}

void swe_sanity_log_destroy(swe_sanity_log *l) try {
    if (!l) return;
    swe_sanity_log_close(l);
    delete l;
} catch (...) {  // no exception crosses the C ABI (allocation, threads)
}

const char *swe_sanity_log_last_error(const swe_sanity_log *l) {
    return l ? l->err.c_str() : "null sanity log";
}

}  // extern "C"
