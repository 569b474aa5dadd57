// nbg_stream.cu -- frame stream writer in the reference's on-disk format.
//
// Format (nbody/nbody_data_stream.cpp:62-160, names at :206-229):
//   <base>.idx   text: "#coord_size 8", "#body_count N", "#box_size B" header
//                lines, then one line per frame "step\ttime\tpart\toffset"
//   <base><k>.dat  frames: N vertices then N velocities, 3 doubles per body;
//                a new part starts when the current one has reached the
//                maximum part size (checked before each frame)
//   <base>.col   N colours, 4 floats per body;  <base>.mass  N doubles
// The header files are written with the first frame, unless the stream
// continues an existing one (append).
//
// GPU form: a frame of engine state is a transpose kernel (SoA y -> the
// frame's AoS layout) and one device-to-host copy into one of two pinned
// buffers, both queued on the engine stream; a host thread waits for the
// copy's event and writes the bytes and the index line.  The caller blocks
// only when both buffers hold frames not yet on disk, so the simulation
// overlaps the file system.  Host frames (already in host memory) go
// through the same thread, synchronously, which keeps frames in order.
#include <sys/stat.h>

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "nbg_internal.cuh"

namespace nbg {
namespace {

// out[0 .. 3N): (x, y, z) per body; out[3N .. 6N): (vx, vy, vz) per body.
__global__ void frame_aos_kernel(const double* __restrict__ y, double* __restrict__ out, size_t n) {
    const size_t total = 6 * n;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total;
         k += (size_t)gridDim.x * blockDim.x) {
        const size_t half = k / (3 * n);  // 0: vertices, 1: velocities
        const size_t r = k - half * 3 * n;
        const size_t body = r / 3, comp = r - body * 3;
        out[k] = y[(half * 3 + comp) * n + body];
    }
}

struct Job {
    int slot = -1;                // pinned slot of a device frame, -1 for a host frame
    const double* host = nullptr; // host frame: 6N doubles in frame layout
    uint64_t step = 0;
    double time = 0.0;
    bool done = false;
    nbg_status status = NBG_OK;
};

}  // namespace
}  // namespace nbg

struct nbg_stream_writer {
    nbg_engine* e = nullptr;  // may be null: host frames only
    std::string base;
    int64_t max_part = 0;
    size_t file_n = 0;
    bool header_written = false;
    bool header_set = false;
    size_t count = 0;
    uint64_t box_size = 0;
    std::vector<float> colors;   // 4 per body
    std::vector<double> mass;
    FILE* dat = nullptr;
    FILE* idx = nullptr;
    std::string last_error;

    // device frames
    double* d_frame = nullptr;
    double* h_pin[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool slot_busy[2] = {false, false};
    int next_slot = 0;

    // writer thread
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<nbg::Job*> queue;
    bool stop = false;
    nbg_status sticky = NBG_OK;  // first error of an asynchronous frame
};

namespace nbg {
namespace {

nbg_status wset(nbg_stream_writer* w, nbg_status s, const char* fmt, const std::string& arg) {
    char buf[512];
    snprintf(buf, sizeof(buf), fmt, arg.c_str());
    w->last_error = buf;
    return s;
}

std::string dat_name(const std::string& base, size_t n) { return base + std::to_string(n) + ".dat"; }

nbg_status open_dat(nbg_stream_writer* w, bool append) {
    if (w->dat) fclose(w->dat);
    const std::string name = dat_name(w->base, w->file_n);
    w->dat = fopen(name.c_str(), append ? "ab" : "wb");
    if (w->dat == nullptr) return wset(w, NBG_ERR_INVALID_ARG, "cannot open %s", name);
    return NBG_OK;
}

nbg_status write_header(nbg_stream_writer* w) {
    fprintf(w->idx, "#coord_size %zu\n#body_count %zu\n#box_size %llu\n", sizeof(double), w->count,
            (unsigned long long)w->box_size);
    const std::string col = w->base + ".col", mass = w->base + ".mass";
    FILE* fc = fopen(col.c_str(), "wb");
    if (fc == nullptr) return wset(w, NBG_ERR_INVALID_ARG, "cannot open %s", col);
    const size_t nc = fwrite(w->colors.data(), sizeof(float), w->colors.size(), fc);
    fclose(fc);
    if (nc != w->colors.size()) return wset(w, NBG_ERR_INVALID_ARG, "cannot write %s", col);
    FILE* fm = fopen(mass.c_str(), "wb");
    if (fm == nullptr) return wset(w, NBG_ERR_INVALID_ARG, "cannot open %s", mass);
    const size_t nm = fwrite(w->mass.data(), sizeof(double), w->mass.size(), fm);
    fclose(fm);
    if (nm != w->mass.size()) return wset(w, NBG_ERR_INVALID_ARG, "cannot write %s", mass);
    w->header_written = true;
    return NBG_OK;
}

// One frame to disk (writer thread): part rollover, bytes, index line.
nbg_status write_frame(nbg_stream_writer* w, const double* frame, uint64_t step, double time) {
    if (!w->header_written) {
        nbg_status s = write_header(w);
        if (s != NBG_OK) return s;
    }
    const long pos0 = ftell(w->dat);
    if (w->max_part > 0 && pos0 >= w->max_part) {
        ++w->file_n;
        nbg_status s = open_dat(w, false);
        if (s != NBG_OK) return s;
    }
    const long fpos = ftell(w->dat);
    const size_t nd = 6 * w->count;
    if (fwrite(frame, sizeof(double), nd, w->dat) != nd || fflush(w->dat) != 0)
        return wset(w, NBG_ERR_INVALID_ARG, "cannot write %s", dat_name(w->base, w->file_n));
    fprintf(w->idx, "%llu\t%g\t%zu\t%ld\n", (unsigned long long)step, time, w->file_n, fpos);
    fflush(w->idx);
    return NBG_OK;
}

void worker_main(nbg_stream_writer* w) {
    if (w->e) cudaSetDevice(w->e->device);
    while (true) {
        Job* job = nullptr;
        {
            std::unique_lock<std::mutex> lk(w->mu);
            w->cv.wait(lk, [&] { return w->stop || !w->queue.empty(); });
            if (w->queue.empty()) return;  // stop requested and nothing left
            job = w->queue.front();
            w->queue.pop_front();
        }
        nbg_status st = NBG_OK;
        const double* frame = job->host;
        if (job->slot >= 0) {
            cudaError_t ce = cudaEventSynchronize(w->ev[job->slot]);
            if (ce != cudaSuccess) {
                st = NBG_ERR_CUDA;
                std::lock_guard<std::mutex> lk(w->mu);
                w->last_error = std::string("frame copy failed: ") + cudaGetErrorString(ce);
            }
            frame = w->h_pin[job->slot];
        }
        if (st == NBG_OK) st = write_frame(w, frame, job->step, job->time);
        {
            std::lock_guard<std::mutex> lk(w->mu);
            if (job->slot >= 0) {
                w->slot_busy[job->slot] = false;
                if (st != NBG_OK && w->sticky == NBG_OK) w->sticky = st;
                delete job;  // nobody waits on a device frame
            } else {
                job->status = st;
                job->done = true;  // the caller owns and frees it
            }
        }
        w->cv.notify_all();
    }
}

nbg_status wait_idle(nbg_stream_writer* w) {
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return w->queue.empty() && !w->slot_busy[0] && !w->slot_busy[1]; });
    const nbg_status s = w->sticky;
    w->sticky = NBG_OK;
    return s;
}

nbg_status take_sticky(nbg_stream_writer* w) {
    std::lock_guard<std::mutex> lk(w->mu);
    const nbg_status s = w->sticky;
    w->sticky = NBG_OK;
    return s;
}

// Last part number of an existing stream (the third field of its last
// frame line), as nbody_data_stream_reader::get_last_file_n gives it.
bool last_part_of(const std::string& idx_name, size_t* part) {
    FILE* f = fopen(idx_name.c_str(), "rb");
    if (f == nullptr) return false;
    char line[512];
    bool any = false;
    while (fgets(line, sizeof(line), f)) {
        if (line[0] == '#') continue;
        unsigned long long s = 0, p = 0;
        double t = 0.0;
        long long off = 0;
        if (sscanf(line, "%llu\t%lf\t%llu\t%lld", &s, &t, &p, &off) == 4) {
            *part = (size_t)p;
            any = true;
        }
    }
    fclose(f);
    return any;
}

void release(nbg_stream_writer* w) {
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->stop = true;
    }
    w->cv.notify_all();
    if (w->worker.joinable()) w->worker.join();
    if (w->dat) fclose(w->dat);
    if (w->idx) fclose(w->idx);
    w->dat = w->idx = nullptr;
    if (w->e) {
        cudaSetDevice(w->e->device);
        cudaFree(w->d_frame);
        for (int s = 0; s < 2; ++s) {
            if (w->h_pin[s]) cudaFreeHost(w->h_pin[s]);
            if (w->ev[s]) cudaEventDestroy(w->ev[s]);
        }
    }
}

}  // namespace
}  // namespace nbg

extern "C" {

nbg_status nbg_stream_open(nbg_engine* e, const char* base_name, int64_t max_part_size, int append,
                           nbg_stream_writer** out) {
    using namespace nbg;
    if (out == nullptr || base_name == nullptr || base_name[0] == '\0') return NBG_ERR_INVALID_ARG;
    *out = nullptr;
    nbg_stream_writer* w = new (std::nothrow) nbg_stream_writer();
    if (w == nullptr) return NBG_ERR_OUT_OF_MEMORY;
    w->e = e;
    w->base = base_name;
    w->max_part = max_part_size;
    // the directory of the base name, made as nbody_data_stream::open does
    const size_t slash = w->base.find_last_of('/');
    if (slash != std::string::npos && slash > 0) {
        const std::string dir = w->base.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0777);  // EEXIST is fine
    }
    if (append != 0) {
        size_t part = 0;
        if (!last_part_of(w->base + ".idx", &part)) {
            delete w;
            return NBG_ERR_INVALID_ARG;
        }
        w->file_n = part;
        w->header_written = true;
    }
    nbg_status s = open_dat(w, append != 0);
    if (s == NBG_OK) {
        const std::string idx = w->base + ".idx";
        w->idx = fopen(idx.c_str(), append != 0 ? "ab" : "wb");
        if (w->idx == nullptr) s = NBG_ERR_INVALID_ARG;
    }
    if (s != NBG_OK) {
        release(w);
        delete w;
        return s;
    }
    w->worker = std::thread(worker_main, w);
    *out = w;
    return NBG_OK;
}

nbg_status nbg_stream_set_header(nbg_stream_writer* w, size_t count, uint64_t box_size,
                                 const float* colors, const double* mass) {
    if (w == nullptr || count == 0 || mass == nullptr) return NBG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(w->mu);
    w->count = count;
    w->box_size = box_size;
    w->colors.assign(4 * count, 0.f);
    if (colors) std::memcpy(w->colors.data(), colors, 4 * count * sizeof(float));
    w->mass.assign(mass, mass + count);
    w->header_set = true;
    return NBG_OK;
}

nbg_status nbg_stream_write(nbg_stream_writer* w, const nbg_buffer* y, uint64_t step, double time) {
    using namespace nbg;
    if (w == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_engine* e = w->e;
    if (e == nullptr) return wset(w, NBG_ERR_INVALID_ARG, "%s", "writer has no engine");
    if (y == nullptr || e->buffers.count(y) == 0)
        return wset(w, NBG_ERR_FOREIGN_BUFFER, "%s", "y is not a buffer of the writer's engine");
    if (!w->header_set) return wset(w, NBG_ERR_NOT_INITIALIZED, "%s", "header not set");
    if (w->count != e->count || y->bytes < 6 * w->count * sizeof(double))
        return wset(w, NBG_ERR_SIZE_MISMATCH, "%s", "frame size differs from the header");
    nbg_status st = take_sticky(w);
    if (st != NBG_OK) return st;
    NBG_CUDA(e, cudaSetDevice(e->device));
    const size_t bytes = 6 * w->count * sizeof(double);
    if (w->d_frame == nullptr) {
        NBG_CUDA(e, cudaMalloc(&w->d_frame, bytes));
        for (int s = 0; s < 2; ++s) {
            NBG_CUDA(e, cudaHostAlloc(reinterpret_cast<void**>(&w->h_pin[s]), bytes,
                                      cudaHostAllocDefault));
            NBG_CUDA(e, cudaEventCreateWithFlags(&w->ev[s], cudaEventDisableTiming));
        }
    }
    const int slot = w->next_slot;
    {
        std::unique_lock<std::mutex> lk(w->mu);
        w->cv.wait(lk, [&] { return !w->slot_busy[slot]; });
        w->slot_busy[slot] = true;
    }
    frame_aos_kernel<<<grid_for(6 * w->count, 256, (unsigned)e->sm_count * 8u), 256, 0, e->stream>>>(
        static_cast<const double*>(y->dptr), w->d_frame, w->count);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(w->h_pin[slot], w->d_frame, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaEventRecord(w->ev[slot], e->stream);
    if (ce != cudaSuccess) {
        std::lock_guard<std::mutex> lk(w->mu);
        w->slot_busy[slot] = false;
        return cuda_error(e, ce, "stream frame copy");
    }
    e->launches++;
    Job* job = new Job();
    job->slot = slot;
    job->step = step;
    job->time = time;
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->queue.push_back(job);
    }
    w->cv.notify_all();
    w->next_slot ^= 1;
    return NBG_OK;
}

nbg_status nbg_stream_write_host(nbg_stream_writer* w, const double* vertices,
                                 const double* velocities, uint64_t step, double time) {
    using namespace nbg;
    if (w == nullptr || vertices == nullptr || velocities == nullptr) return NBG_ERR_INVALID_ARG;
    if (!w->header_set) return wset(w, NBG_ERR_NOT_INITIALIZED, "%s", "header not set");
    std::vector<double> frame(6 * w->count);
    std::memcpy(frame.data(), vertices, 3 * w->count * sizeof(double));
    std::memcpy(frame.data() + 3 * w->count, velocities, 3 * w->count * sizeof(double));
    Job job;
    job.host = frame.data();
    job.step = step;
    job.time = time;
    {
        std::lock_guard<std::mutex> lk(w->mu);
        w->queue.push_back(&job);
    }
    w->cv.notify_all();
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return job.done; });
    const nbg_status s = w->sticky != NBG_OK ? w->sticky : job.status;
    w->sticky = NBG_OK;
    return s;
}

nbg_status nbg_stream_flush(nbg_stream_writer* w) {
    if (w == nullptr) return NBG_ERR_INVALID_ARG;
    return nbg::wait_idle(w);
}

nbg_status nbg_stream_close(nbg_stream_writer* w) {
    if (w == nullptr) return NBG_ERR_INVALID_ARG;
    const nbg_status s = nbg::wait_idle(w);
    nbg::release(w);
    delete w;
    return s;
}

const char* nbg_stream_last_error(const nbg_stream_writer* w) {
    return w == nullptr ? "null writer" : w->last_error.c_str();
}

}  // extern "C"
