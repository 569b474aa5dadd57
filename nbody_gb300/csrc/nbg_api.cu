// nbg_api.cu -- the C ABI of the engine: handles, buffers, argument checks
// and dispatch to the kernels.  Mirrors nbody_engine (nbody/nbody_engine.h)
// with status codes in place of qDebug + return / CUDACHECK exit(3).
#include <cstdarg>
#include <cstring>
#include <new>

#include "nbg_internal.cuh"

namespace nbg {

nbg_status set_error(nbg_engine* e, nbg_status s, const char* fmt, ...) {
    if (e != nullptr) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        e->last_error = buf;
    }
    return s;
}

nbg_status cuda_error(nbg_engine* e, cudaError_t err, const char* what) {
    return set_error(e, NBG_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(err),
                     cudaGetErrorString(err));
}

void prof_begin(nbg_engine* e, int kid, cudaEvent_t* ev) {
    *ev = nullptr;
    if (!e->profiling) return;
    if (e->event_pool.empty()) {
        cudaEvent_t a;
        if (cudaEventCreate(&a) != cudaSuccess) return;
        e->event_pool.push_back(a);
    }
    *ev = e->event_pool.back();
    e->event_pool.pop_back();
    cudaEventRecord(*ev, e->stream);
    (void)kid;
}

void prof_end(nbg_engine* e, int kid, cudaEvent_t ev) {
    if (!e->profiling || ev == nullptr) return;
    cudaEvent_t b;
    if (e->event_pool.empty()) {
        if (cudaEventCreate(&b) != cudaSuccess) return;
    } else {
        b = e->event_pool.back();
        e->event_pool.pop_back();
    }
    cudaEventRecord(b, e->stream);
    e->prof[kid].pending.emplace_back(ev, b);
}

void prof_collect(nbg_engine* e) {
    for (auto& p : e->prof) {
        for (auto& ab : p.pending) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ab.first, ab.second) == cudaSuccess) {
                p.ms += ms;
                p.launches++;
            }
            e->event_pool.push_back(ab.first);
            e->event_pool.push_back(ab.second);
        }
        p.pending.clear();
    }
}

}  // namespace nbg

using namespace nbg;

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static bool own(const nbg_engine* e, const nbg_buffer* b) {
    return b != nullptr && e->buffers.count(b) != 0 && b->magic == kBufferMagic &&
           b->owner == e;
}

static nbg_status check_buf(nbg_engine* e, const nbg_buffer* b, const char* name) {
    if (b == nullptr) return set_error(e, NBG_ERR_INVALID_ARG, "%s is NULL", name);
    if (!own(e, b))
        return set_error(e, NBG_ERR_FOREIGN_BUFFER, "%s is not gb300 memory", name);
    return NBG_OK;
}

static nbg_status collect_terms(nbg_engine* e, const nbg_buffer* const* b, size_t bcount,
                                const double* c, size_t csize, size_t need_bytes,
                                std::vector<const double*>* ptrs,
                                std::vector<double>* coef) {
    if (csize > bcount)
        return set_error(e, NBG_ERR_INVALID_ARG, "csize > b.size()");
    if (csize > 0 && b == nullptr) return set_error(e, NBG_ERR_INVALID_ARG, "b is NULL");
    for (size_t k = 0; k < csize; ++k) {
        nbg_status s = check_buf(e, b[k], "b[k]");
        if (s != NBG_OK) return s;
        if (b[k]->bytes < need_bytes)
            return set_error(e, NBG_ERR_SIZE_MISMATCH, "b[%zu] smaller than a", k);
    }
    for (size_t k = 0; k < csize; ++k) {
        if (c[k] == 0.0) continue;  // nbody/nbody_engine.cpp:58-61
        ptrs->push_back(static_cast<const double*>(b[k]->dptr));
        coef->push_back(c[k]);
    }
    return NBG_OK;
}

static nbg_status sync_and_check(nbg_engine* e) {
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    prof_collect(e);
    if (*e->h_err != 0) {
        unsigned bits = *e->h_err;
        *e->h_err = 0;
        if (bits & kDevErrTimeout)
            return set_error(e, NBG_ERR_DEVICE_TIMEOUT,
                             "a device-side wait timed out (error bits 0x%x)", bits);
        return set_error(e, NBG_ERR_DEVICE_ERROR, "kernel error flag 0x%x", bits);
    }
    return NBG_OK;
}

// Queue a copy of the device error word into pinned memory (read at sync).
static nbg_status queue_err_readback(nbg_engine* e) {
    NBG_CUDA(e, cudaMemcpyAsync(e->h_err, e->d_err, sizeof(unsigned),
                                cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(e, cudaMemsetAsync(e->d_err, 0, sizeof(unsigned), e->stream));
    return NBG_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void nbg_params_default(nbg_params* p) {
    if (p == nullptr) return;
    memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(nbg_params);
    p->device = 0;
    p->algo = NBG_ALGO_DIRECT;
    p->precision = NBG_PREC_FP64;
    p->softening = 0.0;
    p->distance_to_node_radius_ratio = 10.0;  // nbody/nbody_engines.cpp:44
    p->tree_build_rate = 0;
    p->tree_layout = NBG_LAYOUT_HEAP_STACKLESS;
    p->traverse_type = NBG_TRAVERSE_NESTED_TREE;
    p->learned = 0;
    p->block_size = 0;
    p->learned_tight_ratio = 2.0;
}

int nbg_abi_version(void) { return NBG_ABI_VERSION; }

const char* nbg_status_string(nbg_status s) {
    switch (s) {
        case NBG_OK: return "ok";
        case NBG_ERR_INVALID_ARG: return "invalid argument";
        case NBG_ERR_FOREIGN_BUFFER: return "foreign buffer";
        case NBG_ERR_SIZE_MISMATCH: return "size mismatch";
        case NBG_ERR_OUT_OF_MEMORY: return "out of memory";
        case NBG_ERR_CUDA: return "cuda error";
        case NBG_ERR_UNSUPPORTED: return "unsupported";
        case NBG_ERR_NOT_INITIALIZED: return "not initialized";
        case NBG_ERR_DEVICE_TIMEOUT: return "device timeout";
        case NBG_ERR_DEVICE_ERROR: return "device error";
        case NBG_ERR_TOO_LARGE: return "exceeds a fixed capacity";
    }
    return "unknown";
}

nbg_status nbg_engine_create(const nbg_params* p, nbg_engine** out) {
    if (out == nullptr) return NBG_ERR_INVALID_ARG;
    *out = nullptr;
    nbg_params prm;
    nbg_params_default(&prm);
    if (p != nullptr) {
        if (p->struct_size != sizeof(nbg_params)) return NBG_ERR_INVALID_ARG;
        prm = *p;
    }
    if (prm.algo != NBG_ALGO_DIRECT && prm.algo != NBG_ALGO_BH) return NBG_ERR_INVALID_ARG;
    if (prm.precision != NBG_PREC_FP64 && prm.precision != NBG_PREC_MIXED)
        return NBG_ERR_INVALID_ARG;
    if (!(prm.softening >= 0.0)) return NBG_ERR_INVALID_ARG;
    if (prm.block_size < 0) return NBG_ERR_INVALID_ARG;
    if (prm.algo == NBG_ALGO_BH) {
        if (prm.tree_layout != NBG_LAYOUT_HEAP && prm.tree_layout != NBG_LAYOUT_HEAP_STACKLESS)
            return NBG_ERR_INVALID_ARG;
        if (prm.traverse_type != NBG_TRAVERSE_CYCLE &&
            prm.traverse_type != NBG_TRAVERSE_NESTED_TREE)
            return NBG_ERR_INVALID_ARG;
        if (!(prm.distance_to_node_radius_ratio > 0.0)) return NBG_ERR_INVALID_ARG;
        if (prm.learned && prm.precision != NBG_PREC_MIXED) return NBG_ERR_INVALID_ARG;
    } else if (prm.learned) {
        return NBG_ERR_INVALID_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return NBG_ERR_CUDA;
    if (prm.device < 0 || prm.device >= ndev) return NBG_ERR_INVALID_ARG;

    nbg_engine* e = new (std::nothrow) nbg_engine();
    if (e == nullptr) return NBG_ERR_OUT_OF_MEMORY;
    e->params = prm;
    e->device = prm.device;
    if (cudaSetDevice(e->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, e->device) !=
            cudaSuccess ||
        cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&e->d_scalar, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&e->d_err, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(e->d_err, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaHostAlloc(&e->h_scalar, 2 * sizeof(double), cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc(&e->h_err, sizeof(unsigned), cudaHostAllocDefault) != cudaSuccess) {
        nbg_engine_destroy(e);
        return NBG_ERR_CUDA;
    }
    *e->h_err = 0;
    *out = e;
    return NBG_OK;
}

void nbg_engine_destroy(nbg_engine* e) {
    if (e == nullptr) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    tree_destroy(e);
    learn_destroy(e);
    judge_destroy(e);
    for (const nbg_buffer* b : e->buffers) {
        cudaFree(b->dptr);
        delete b;
    }
    e->buffers.clear();
    cudaFree(e->d_mass);
    cudaFree(e->d_massf);
    cudaFree(e->d_xyzm);
    cudaFree(e->d_scalar);
    cudaFree(e->d_err);
    if (e->h_scalar) cudaFreeHost(e->h_scalar);
    if (e->h_err) cudaFreeHost(e->h_err);
    for (auto& p : e->prof)
        for (auto& ab : p.pending) {
            cudaEventDestroy(ab.first);
            cudaEventDestroy(ab.second);
        }
    for (cudaEvent_t ev : e->event_pool) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* nbg_type_name(const nbg_engine* e) {
    if (e == nullptr) return "nbody_engine_gb300";
    if (e->params.algo == NBG_ALGO_BH) return "nbody_engine_gb300_bh";
    return "nbody_engine_gb300";
}

const char* nbg_last_error(const nbg_engine* e) {
    return e == nullptr ? "" : e->last_error.c_str();
}

nbg_status nbg_create_buffer(nbg_engine* e, size_t bytes, nbg_buffer** out) {
    if (e == nullptr || out == nullptr) return NBG_ERR_INVALID_ARG;
    *out = nullptr;
    NBG_CUDA(e, cudaSetDevice(e->device));
    nbg_buffer* b = new (std::nothrow) nbg_buffer();
    if (b == nullptr) return set_error(e, NBG_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->magic = kBufferMagic;
    b->owner = e;
    b->bytes = bytes;
    b->dptr = nullptr;
    // Round up so vector kernels may touch whole 16-byte words; never read
    // past bytes.  A zero-byte buffer still gets a valid address.
    size_t alloc = (bytes + 255) & ~size_t(255);
    if (alloc == 0) alloc = 256;
    cudaError_t err = cudaMalloc(&b->dptr, alloc);
    if (err != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return set_error(e, NBG_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu) failed: %s", bytes,
                         cudaGetErrorString(err));
    }
    e->buffers.insert(b);
    *out = b;
    return NBG_OK;
}

nbg_status nbg_free_buffer(nbg_engine* e, nbg_buffer* b) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (b == nullptr) return NBG_OK;  // delete NULL is a no-op in the reference
    nbg_status s = check_buf(e, b, "buffer");
    if (s != NBG_OK) return s;
    if (b == e->y) return set_error(e, NBG_ERR_INVALID_ARG, "y is owned by the engine");
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    e->buffers.erase(b);
    b->magic = 0;
    cudaFree(b->dptr);
    delete b;
    return NBG_OK;
}

size_t nbg_buffer_size(const nbg_buffer* b) {
    return (b != nullptr && b->magic == kBufferMagic) ? b->bytes : 0;
}

void* nbg_buffer_device_ptr(nbg_buffer* b) {
    return (b != nullptr && b->magic == kBufferMagic) ? b->dptr : nullptr;
}

nbg_status nbg_init(nbg_engine* e, size_t count, const double* vertices,
                    const double* velocities, const double* mass) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (count == 0 || vertices == nullptr || velocities == nullptr || mass == nullptr)
        return set_error(e, NBG_ERR_INVALID_ARG, "init: empty or NULL data");
    if (e->params.algo == NBG_ALGO_BH && (count & (count - 1)) != 0)
        return set_error(e, NBG_ERR_UNSUPPORTED,
                         "Barnes-Hut needs a power-of-two body count (heap leaves at "
                         "[N, 2N)), got %zu",
                         count);
    NBG_CUDA(e, cudaSetDevice(e->device));
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    if (e->y != nullptr) {
        e->buffers.erase(e->y);
        cudaFree(e->y->dptr);
        delete e->y;
        e->y = nullptr;
    }
    cudaFree(e->d_mass);
    cudaFree(e->d_massf);
    e->d_mass = nullptr;
    e->d_massf = nullptr;
    tree_destroy(e);
    e->count = count;
    nbg_buffer* y = nullptr;
    nbg_status s = nbg_create_buffer(e, 6 * count * sizeof(double), &y);
    if (s != NBG_OK) return s;
    e->y = y;
    NBG_CUDA(e, cudaMalloc(&e->d_mass, count * sizeof(double)));
    NBG_CUDA(e, cudaMalloc(&e->d_massf, count * sizeof(float)));
    // AoS -> SoA on the host, then one copy (init is not on the hot path).
    std::vector<double> h(6 * count);
    for (size_t i = 0; i < count; ++i)
        for (int d = 0; d < 3; ++d) {
            h[d * count + i] = vertices[3 * i + d];
            h[(3 + d) * count + i] = velocities[3 * i + d];
        }
    std::vector<float> mf(count);
    for (size_t i = 0; i < count; ++i) mf[i] = (float)mass[i];
    // equal masses (a common initial condition) let the mixed direct kernel
    // scale the pair sums by the mass once instead of weighting every pair
    e->uniform_mass = true;
    for (size_t i = 1; i < count && e->uniform_mass; ++i) e->uniform_mass = mass[i] == mass[0];
    e->mass_value = mass[0];
    NBG_CUDA(e, cudaMemcpy(y->dptr, h.data(), 6 * count * sizeof(double),
                           cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(e->d_mass, mass, count * sizeof(double), cudaMemcpyHostToDevice));
    NBG_CUDA(e, cudaMemcpy(e->d_massf, mf.data(), count * sizeof(float),
                           cudaMemcpyHostToDevice));
    return NBG_OK;
}

nbg_status nbg_get_data(nbg_engine* e, double* vertices, double* velocities) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (e->y == nullptr) return set_error(e, NBG_ERR_NOT_INITIALIZED, "engine not initialized");
    if (vertices == nullptr || velocities == nullptr)
        return set_error(e, NBG_ERR_INVALID_ARG, "get_data: NULL output");
    size_t n = e->count;
    std::vector<double> h(6 * n);
    NBG_CUDA(e, cudaMemcpyAsync(h.data(), e->y->dptr, 6 * n * sizeof(double),
                                cudaMemcpyDeviceToHost, e->stream));
    nbg_status s = sync_and_check(e);
    if (s != NBG_OK) return s;
    for (size_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            vertices[3 * i + d] = h[d * n + i];
            velocities[3 * i + d] = h[(3 + d) * n + i];
        }
    return NBG_OK;
}

size_t nbg_problem_size(const nbg_engine* e) { return e == nullptr ? 0 : 6 * e->count; }

nbg_buffer* nbg_get_y(nbg_engine* e) { return e == nullptr ? nullptr : e->y; }

nbg_status nbg_fcompute(nbg_engine* e, double t, uint64_t step, const nbg_buffer* y,
                        nbg_buffer* f) {
    (void)t;  // unused by every reference engine
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, y, "y");
    if (s != NBG_OK) return s;
    s = check_buf(e, f, "f");
    if (s != NBG_OK) return s;
    if (e->count == 0) return set_error(e, NBG_ERR_NOT_INITIALIZED, "engine not initialized");
    size_t need = 6 * e->count * sizeof(double);
    if (y->bytes < need || f->bytes < need)
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "fcompute: y/f smaller than 6N doubles");
    if (y == f) return set_error(e, NBG_ERR_INVALID_ARG, "fcompute: y and f alias");
    NBG_CUDA(e, cudaSetDevice(e->device));
    const double* yd = static_cast<const double*>(y->dptr);
    double* fd = static_cast<double*>(f->dptr);
    if (e->params.algo == NBG_ALGO_BH) return bh_fcompute(e, step, yd, fd);
    return direct_fcompute(e, yd, fd);
}

nbg_status nbg_clamp(nbg_engine* e, nbg_buffer* y, double b) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, y, "y");
    if (s != NBG_OK) return s;
    if (e->count == 0) return set_error(e, NBG_ERR_NOT_INITIALIZED, "engine not initialized");
    if (y->bytes < 3 * e->count * sizeof(double))
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "clamp: y too small");
    return launch_clamp(e, static_cast<double*>(y->dptr), b, 3 * e->count);
}

nbg_status nbg_read_buffer(nbg_engine* e, void* dst, const nbg_buffer* src) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, src, "src");
    if (s != NBG_OK) return s;
    if (dst == nullptr && src->bytes > 0)
        return set_error(e, NBG_ERR_INVALID_ARG, "read_buffer: dst is NULL");
    if (src->bytes > 0)
        NBG_CUDA(e, cudaMemcpyAsync(dst, src->dptr, src->bytes, cudaMemcpyDeviceToHost,
                                    e->stream));
    s = queue_err_readback(e);
    if (s != NBG_OK) return s;
    return sync_and_check(e);
}

nbg_status nbg_write_buffer(nbg_engine* e, nbg_buffer* dst, const void* src) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, dst, "dst");
    if (s != NBG_OK) return s;
    if (src == nullptr && dst->bytes > 0)
        return set_error(e, NBG_ERR_INVALID_ARG, "write_buffer: src is NULL");
    if (dst->bytes > 0)
        NBG_CUDA(e, cudaMemcpyAsync(dst->dptr, src, dst->bytes, cudaMemcpyHostToDevice,
                                    e->stream));
    // The reference synchronizes after the copy (nbody_engine_cuda.cpp:312); the
    // caller may reuse src as soon as this returns.
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    return NBG_OK;
}

nbg_status nbg_copy_buffer(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    s = check_buf(e, b, "b");
    if (s != NBG_OK) return s;
    if (a->bytes != b->bytes)
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "Size does not match");
    if (a != b && a->bytes > 0)
        NBG_CUDA(e, cudaMemcpyAsync(a->dptr, b->dptr, a->bytes, cudaMemcpyDeviceToDevice,
                                    e->stream));
    return NBG_OK;
}

nbg_status nbg_fill_buffer(nbg_engine* e, nbg_buffer* a, double value) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    return launch_fill(e, static_cast<double*>(a->dptr), value, a->bytes / sizeof(double));
}

nbg_status nbg_fmadd_inplace(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b, double c) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    s = check_buf(e, b, "b");
    if (s != NBG_OK) return s;
    if (b->bytes < a->bytes) return set_error(e, NBG_ERR_SIZE_MISMATCH, "b smaller than a");
    Terms t{};
    t.k = 1;
    t.p[0] = static_cast<const double*>(b->dptr);
    t.c[0] = c;
    return launch_axpy_n(e, static_cast<double*>(a->dptr), nullptr, kBaseSelf, t,
                         a->bytes / sizeof(double));
}

nbg_status nbg_fmadd(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b, const nbg_buffer* c,
                     double d) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    s = check_buf(e, b, "b");
    if (s != NBG_OK) return s;
    s = check_buf(e, c, "c");
    if (s != NBG_OK) return s;
    if (b->bytes < a->bytes || c->bytes < a->bytes)
        return set_error(e, NBG_ERR_SIZE_MISMATCH, "b or c smaller than a");
    Terms t{};
    t.k = 1;
    t.p[0] = static_cast<const double*>(c->dptr);
    t.c[0] = d;
    return launch_axpy_n(e, static_cast<double*>(a->dptr), static_cast<const double*>(b->dptr),
                         kBasePtr, t, a->bytes / sizeof(double));
}

static nbg_status run_terms(nbg_engine* e, double* a, const double* base, int mode,
                            const std::vector<const double*>& p, const std::vector<double>& c,
                            size_t n) {
    // One fused pass per 16 terms; the first pass starts from the requested
    // base, later passes accumulate onto a.
    size_t k0 = 0;
    bool first = true;
    do {
        Terms t{};
        t.k = 0;
        for (; k0 < p.size() && t.k < Terms::kMax; ++k0, ++t.k) {
            t.p[t.k] = p[k0];
            t.c[t.k] = c[k0];
        }
        nbg_status s = launch_axpy_n(e, a, base, first ? mode : (int)kBaseSelf, t, n);
        if (s != NBG_OK) return s;
        first = false;
    } while (k0 < p.size());
    return NBG_OK;
}

nbg_status nbg_fmaddn_inplace(nbg_engine* e, nbg_buffer* a, const nbg_buffer* const* b,
                              size_t bcount, const double* c, size_t csize) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (c == nullptr) return NBG_OK;  // nbody/nbody_engine.cpp:49-52
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    std::vector<const double*> p;
    std::vector<double> cc;
    s = collect_terms(e, b, bcount, c, csize, a->bytes, &p, &cc);
    if (s != NBG_OK) return s;
    if (p.empty()) return NBG_OK;
    return run_terms(e, static_cast<double*>(a->dptr), nullptr, kBaseSelf, p, cc,
                     a->bytes / sizeof(double));
}

nbg_status nbg_fmaddn_corr(nbg_engine* e, nbg_buffer* a, nbg_buffer* corr,
                           const nbg_buffer* const* b, size_t bcount, const double* c,
                           size_t csize) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    s = check_buf(e, corr, "corr");
    if (s != NBG_OK) return s;
    if (c == nullptr) return set_error(e, NBG_ERR_INVALID_ARG, "c must not be nullptr");
    if (corr->bytes < a->bytes) return set_error(e, NBG_ERR_SIZE_MISMATCH, "corr smaller than a");
    std::vector<const double*> p;
    std::vector<double> cc;
    s = collect_terms(e, b, bcount, c, csize, a->bytes, &p, &cc);
    if (s != NBG_OK) return s;
    size_t k0 = 0;
    while (k0 < p.size()) {
        Terms t{};
        t.k = 0;
        for (; k0 < p.size() && t.k < Terms::kMax; ++k0, ++t.k) {
            t.p[t.k] = p[k0];
            t.c[t.k] = cc[k0];
        }
        s = launch_axpy_n_corr(e, static_cast<double*>(a->dptr), static_cast<double*>(corr->dptr),
                               t, a->bytes / sizeof(double));
        if (s != NBG_OK) return s;
    }
    return NBG_OK;
}

nbg_status nbg_fmaddn(nbg_engine* e, nbg_buffer* a, const nbg_buffer* b,
                      const nbg_buffer* const* c, size_t ccount, const double* d,
                      size_t dsize) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    if (d == nullptr) return set_error(e, NBG_ERR_INVALID_ARG, "d == NULL");
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    if (b != nullptr) {
        s = check_buf(e, b, "b");
        if (s != NBG_OK) return s;
        if (b->bytes < a->bytes) return set_error(e, NBG_ERR_SIZE_MISMATCH, "b smaller than a");
    }
    std::vector<const double*> p;
    std::vector<double> cc;
    s = collect_terms(e, c, ccount, d, dsize, a->bytes, &p, &cc);
    if (s != NBG_OK) return s;
    size_t n = a->bytes / sizeof(double);
    double* ad = static_cast<double*>(a->dptr);
    if (b == nullptr) {
        if (p.empty()) return launch_fill(e, ad, 0.0, n);  // nbody/nbody_engine.cpp:91-95
        return run_terms(e, ad, nullptr, kBaseZero, p, cc, n);
    }
    if (p.empty()) return NBG_OK;  // no nonzero term: a untouched (nbody_engine.cpp:97-112)
    return run_terms(e, ad, static_cast<const double*>(b->dptr), kBasePtr, p, cc, n);
}

nbg_status nbg_fmaxabs(nbg_engine* e, const nbg_buffer* a, double* result) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = check_buf(e, a, "a");
    if (s != NBG_OK) return s;
    if (result == nullptr) return set_error(e, NBG_ERR_INVALID_ARG, "result is NULL");
    size_t n = a->bytes / sizeof(double);
    if (n == 0) {
        *result = 0.0;
        return NBG_OK;
    }
    s = launch_maxabs(e, static_cast<const double*>(a->dptr), n);
    if (s != NBG_OK) return s;
    NBG_CUDA(e, cudaMemcpyAsync(e->h_scalar, e->d_scalar, sizeof(double),
                                cudaMemcpyDeviceToHost, e->stream));
    s = queue_err_readback(e);
    if (s != NBG_OK) return s;
    s = sync_and_check(e);
    if (s != NBG_OK) return s;
    *result = e->h_scalar[0];
    return NBG_OK;
}

nbg_status nbg_synchronize(nbg_engine* e) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    nbg_status s = queue_err_readback(e);
    if (s != NBG_OK) return s;
    return sync_and_check(e);
}

void* nbg_stream(nbg_engine* e) { return e == nullptr ? nullptr : (void*)e->stream; }

nbg_status nbg_host_alloc(size_t bytes, void** out) {
    if (out == nullptr) return NBG_ERR_INVALID_ARG;
    *out = nullptr;
    if (cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return NBG_ERR_OUT_OF_MEMORY;
    }
    return NBG_OK;
}

void nbg_host_free(void* p) {
    if (p != nullptr) cudaFreeHost(p);
}

nbg_status nbg_profile_enable(nbg_engine* e, int enable) {
    if (e == nullptr) return NBG_ERR_INVALID_ARG;
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    prof_collect(e);
    e->profiling = enable != 0;
    return NBG_OK;
}

nbg_status nbg_profile_query(nbg_engine* e, int kernel_id, double* total_ms,
                             uint64_t* launches) {
    if (e == nullptr || kernel_id < 0 || kernel_id >= NBG_K_COUNT) return NBG_ERR_INVALID_ARG;
    NBG_CUDA(e, cudaStreamSynchronize(e->stream));
    prof_collect(e);
    if (total_ms) *total_ms = e->prof[kernel_id].ms;
    if (launches) *launches = e->prof[kernel_id].launches;
    e->prof[kernel_id].ms = 0.0;
    e->prof[kernel_id].launches = 0;
    return NBG_OK;
}

uint64_t nbg_launch_count(const nbg_engine* e) { return e == nullptr ? 0 : e->launches; }

nbg_status nbg_tune_set(nbg_engine* e, const char* key, int64_t value) {
    if (e == nullptr || key == nullptr) return NBG_ERR_INVALID_ARG;
    e->tune[key] = value;
    return NBG_OK;
}

nbg_status nbg_tune_get(nbg_engine* e, const char* key, int64_t* value) {
    if (e == nullptr || key == nullptr || value == nullptr) return NBG_ERR_INVALID_ARG;
    auto it = e->tune.find(key);
    if (it == e->tune.end()) return set_error(e, NBG_ERR_INVALID_ARG, "tuning key %s not set", key);
    *value = it->second;
    return NBG_OK;
}

nbg_status nbg_measure_fp32_peak(nbg_engine* e, double* flops) {
    if (e == nullptr || flops == nullptr) return NBG_ERR_INVALID_ARG;
    return measure_fp32_peak(e, flops);
}

}  // extern "C"
