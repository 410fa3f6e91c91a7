// C ABI: particle transfers between host and device (SI FP64 and packed FP32),
// the pipelined step of host-resident populations (pcl_advance_host) and
// page-locked host memory.
#include "ctx_internal.cuh"

using namespace pcl;

extern "C" {

int pcl_upload(void* ctx, int species, int64_t n, const double* x, const double* p, const double* w,
               const double* t, const double* s, const uint64_t* sid, uint64_t sid_base) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (!S.set || S.cap == 0) return fail(c, PCL_ERR_STATE, "species not set or tally-only");
    if (n < 0 || n > S.cap) return fail(c, PCL_ERR_CAPACITY, "upload exceeds capacity");
    if (n > 0 && (!x || !p || !w || !t)) return fail(c, PCL_ERR_INVALID, "null particle arrays");
    std::vector<float4> hx(n), hp(n);
    std::vector<uint4> hm(n);
    const uint32_t k0 = uint32_t(c->cfg.seed), k1 = uint32_t(c->cfg.seed >> 32);
    for (int64_t i = 0; i < n; ++i) {
        uint64_t id = sid ? sid[i] : sid_base + uint64_t(i);
        uint32_t ctr = 0;
        double sv;
        if (s) {
            sv = s[i];
        } else {  // s = nextcoll() drawn from the particle's own stream (electron.jl:30-33)
            uint32_t cc[4] = {0u, uint32_t(id), uint32_t(id >> 32), 0u};
            philox_host(cc, k0, k1);
            double u = double(((cc[0] >> 9) << 1) | 1u) * 5.9604644775390625e-8;
            sv = -std::log(u);
            ctr = 1;
        }
        hx[i] = make_float4(float(x[3 * i]), float(x[3 * i + 1]), float(x[3 * i + 2]), float(w[i]));
        hp[i] = make_float4(float(p_to_dev(p[3 * i])), float(p_to_dev(p[3 * i + 1])),
                            float(p_to_dev(p[3 * i + 2])), float(sv));
        float toff = float(t_to_dev(t[i] - c->t));
        uint32_t tb;
        std::memcpy(&tb, &toff, 4);
        hm[i] = make_uint4(uint32_t(id), uint32_t(id >> 32), ctr, tb);
    }
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (n > 0) {
        CK(h2d(c, S.xw[S.cur], hx.data(), sizeof(float4) * n));
        CK(h2d(c, S.ps[S.cur], hp.data(), sizeof(float4) * n));
        CK(h2d(c, S.meta[S.cur], hm.data(), sizeof(uint4) * n));
    }
    unsigned long long nn = (unsigned long long)n;
    CK(h2d(c, &c->d_ctl->n[species], &nn, sizeof(nn)));
    c->live[species] = n;
    return PCL_OK;
}


int pcl_download(void* ctx, int species, int64_t* n, double* x, double* p, double* w, double* t, double* s,
                 uint64_t* sid, uint32_t* ctr) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    std::vector<float4> hx(slots), hp(slots);
    std::vector<uint4> hm(slots);
    if (slots > 0) {
        CK(d2h(c, hx.data(), S.xw[S.cur], sizeof(float4) * slots));
        CK(d2h(c, hp.data(), S.ps[S.cur], sizeof(float4) * slots));
        CK(d2h(c, hm.data(), S.meta[S.cur], sizeof(uint4) * slots));
    }
    int64_t capn = *n, m = 0;
    for (long long i = 0; i < slots; ++i) {
        if (hm[i].z == PCL_DEAD_CTR) continue;
        if (m >= capn) return fail(c, PCL_ERR_CAPACITY, "download arrays too small");
        if (x) { x[3 * m] = hx[i].x; x[3 * m + 1] = hx[i].y; x[3 * m + 2] = hx[i].z; }
        if (p) {
            p[3 * m] = p_to_si(hp[i].x); p[3 * m + 1] = p_to_si(hp[i].y); p[3 * m + 2] = p_to_si(hp[i].z);
        }
        if (w) w[m] = hx[i].w;
        if (s) s[m] = hp[i].w;
        float toff;
        std::memcpy(&toff, &hm[i].w, 4);
        if (t) t[m] = c->t + t_to_si(toff);
        if (sid) sid[m] = uint64_t(hm[i].x) | (uint64_t(hm[i].y) << 32);
        if (ctr) ctr[m] = hm[i].z;
        ++m;
    }
    *n = m;
    return PCL_OK;
}

int pcl_upload_packed(void* ctx, int species, int64_t n, const pcl_packed* host) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !host) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (!S.set || S.cap == 0) return fail(c, PCL_ERR_STATE, "species not set or tally-only");
    if (n < 0 || n > S.cap) return fail(c, PCL_ERR_CAPACITY, "upload exceeds capacity");
    CK(cudaSetDevice(c->device));
    if (n > 0) {
        CK(cudaMemcpyAsync(S.xw[S.cur], host->xw, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(S.ps[S.cur], host->ps, sizeof(float4) * n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(S.meta[S.cur], host->meta, sizeof(uint4) * n, cudaMemcpyHostToDevice, c->stream));
    }
    unsigned long long nn = (unsigned long long)n;
    CK(cudaMemcpyAsync(&c->d_ctl->n[species], &nn, sizeof(nn), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = n;
    return PCL_OK;
}

int pcl_download_packed(void* ctx, int species, int64_t* n, pcl_packed* host) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !host || !n) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    if (slots > *n) return fail(c, PCL_ERR_CAPACITY, "download arrays too small");
    if (slots > 0) {
        CK(cudaMemcpyAsync(host->xw, S.xw[S.cur], sizeof(float4) * slots, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(host->ps, S.ps[S.cur], sizeof(float4) * slots, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(host->meta, S.meta[S.cur], sizeof(uint4) * slots, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    *n = slots;
    return PCL_OK;
}

// Slots [a, b) of each species covered by concatenated indices [g0, g1) of
// the species ranges n[0], n[1], n[2] (the step kernel's work order).
static void chunk_ranges(const long long n[3], long long g0, long long g1, long long a[3], long long b[3]) {
    long long base = 0;
    for (int s = 0; s < 3; ++s) {
        a[s] = std::min(std::max(g0 - base, 0ll), n[s]);
        b[s] = std::min(std::max(g1 - base, 0ll), n[s]);
        base += n[s];
    }
}

static cudaError_t copy_slots(const SpeciesState& S, const pcl_packed& h, long long a, long long b, bool up,
                              cudaStream_t st) {
    if (b <= a) return cudaSuccess;
    const size_t n = size_t(b - a);
    cudaError_t e;
    if (up) {
        e = cudaMemcpyAsync(S.xw[S.cur] + a, reinterpret_cast<const float4*>(h.xw) + a, 16 * n,
                            cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(S.ps[S.cur] + a, reinterpret_cast<const float4*>(h.ps) + a, 16 * n,
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(S.meta[S.cur] + a, reinterpret_cast<const uint4*>(h.meta) + a, 16 * n,
                                cudaMemcpyHostToDevice, st);
    } else {
        e = cudaMemcpyAsync(reinterpret_cast<float4*>(h.xw) + a, S.xw[S.cur] + a, 16 * n, cudaMemcpyDeviceToHost,
                            st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(reinterpret_cast<float4*>(h.ps) + a, S.ps[S.cur] + a, 16 * n,
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(reinterpret_cast<uint4*>(h.meta) + a, S.meta[S.cur] + a, 16 * n,
                                cudaMemcpyDeviceToHost, st);
    }
    return e;
}

// Device-usable address of page-locked host memory (nullptr: not page-locked
// or not reachable by the device).  Clears the error a failed query leaves.
static void* device_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return at.devicePointer;
}

int pcl_set_host_io(void* ctx, int mode) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (mode < PCL_HOST_IO_AUTO || mode > PCL_HOST_IO_DIRECT) return fail(c, PCL_ERR_INVALID, "host i/o mode");
    c->host_io = mode;
    return PCL_OK;
}

int pcl_advance_host(void* ctx, double tfinal, const int64_t* n_in, const pcl_packed* in, int64_t* n_out,
                     pcl_packed* out, const int64_t* out_cap, int nchunks, int compact) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n_in || !in || !n_out || !out || !out_cap) return PCL_ERR_INVALID;
    if (!(tfinal > c->t)) return fail(c, PCL_ERR_INVALID, "tfinal must exceed the current time");
    if (nchunks < 1 || nchunks > 64) return fail(c, PCL_ERR_INVALID, "nchunks must be in [1, 64]");
    bool any = false;
    long long n[3];
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        any = any || S.set;
        n[s] = (S.set && S.cap > 0) ? (long long)n_in[s] : 0;
        if (n[s] < 0 || n[s] > S.cap) return fail(c, PCL_ERR_CAPACITY, "input exceeds capacity");
        if (n[s] > 0 && (!in[s].xw || !in[s].ps || !in[s].meta))
            return fail(c, PCL_ERR_INVALID, "null input arrays");
        // a species may gain secondaries in the step even if it starts empty
        if (out_cap[s] < 0 || (out_cap[s] > 0 && (!out[s].xw || !out[s].ps || !out[s].meta)))
            return fail(c, PCL_ERR_INVALID, "null or negative-size output arrays");
        if (out_cap[s] < n[s]) return fail(c, PCL_ERR_CAPACITY, "output arrays smaller than the input");
    }
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    // host-direct mode: every array the kernels would touch must be page-locked
    // and usable by the device
    bool direct = c->host_io == PCL_HOST_IO_DIRECT;
    void* hv[3][6] = {};
    for (int s = 0; s < 3 && direct; ++s) {
        if (n[s] > 0) {
            hv[s][0] = device_view(in[s].xw); hv[s][1] = device_view(in[s].ps); hv[s][2] = device_view(in[s].meta);
            direct = hv[s][0] && hv[s][1] && hv[s][2];
        }
        if (direct && out_cap[s] > 0) {
            hv[s][3] = device_view(out[s].xw); hv[s][4] = device_view(out[s].ps); hv[s][5] = device_view(out[s].meta);
            direct = hv[s][3] && hv[s][4] && hv[s][5];
        }
    }
    if (c->host_io == PCL_HOST_IO_DIRECT && !direct)
        return fail(c, PCL_ERR_INVALID, "host-direct mode needs page-locked arrays the device can use");
    // every return, error or not, leaves no copy or kernel using the caller's
    // buffers in flight, and the host-direct pointers cleared
    struct Drain {
        Ctx* c;
        ~Drain() {
            if (c->s_h2d) cudaStreamSynchronize(c->s_h2d);
            if (c->s_d2h) cudaStreamSynchronize(c->s_d2h);
            if (c->s_cmp) cudaStreamSynchronize(c->s_cmp);
            cudaStreamSynchronize(c->stream);
            for (int s = 0; s < 3; ++s) {
                c->hin_xw[s] = nullptr; c->hin_ps[s] = nullptr; c->hin_meta[s] = nullptr;
                c->hx_xw[s] = nullptr; c->hx_ps[s] = nullptr; c->hx_meta[s] = nullptr;
                c->hx_cap[s] = 0;
            }
        }
    } drain{c};
    int rc = build_blob(c);
    if (rc || (rc = ensure_spill(c)) || (rc = ensure_lq(c))) return rc;
    if (!c->s_h2d) CK(cudaStreamCreateWithFlags(&c->s_h2d, cudaStreamNonBlocking));
    if (!c->s_d2h) CK(cudaStreamCreateWithFlags(&c->s_d2h, cudaStreamNonBlocking));
    if (!c->s_cmp) CK(cudaStreamCreateWithFlags(&c->s_cmp, cudaStreamNonBlocking));
    if (!c->io_join) CK(cudaEventCreateWithFlags(&c->io_join, cudaEventDisableTiming));
    if (!c->d_heads) CK(cudaMalloc(&c->d_heads, 64 * sizeof(unsigned long long)));
    while ((int)c->io_ev.size() < 2 * nchunks) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->io_ev.push_back(e);
        CK(cudaEventCreate(&e));
        c->io_tev.push_back(e);
    }
    const double dt_si = tfinal - c->t;
    const double dt = t_to_dev(dt_si);
    const int threads = block_threads(c);
    const size_t smem = step_smem_bytes(int(c->blob.size()), threads, c->cfg.classic_step == 0);
    const int minb = blocks_per_sm(c);
    // slot counts, then the step prologue (k_begin takes n_start from them)
    unsigned long long nn[3] = {(unsigned long long)n[0], (unsigned long long)n[1], (unsigned long long)n[2]};
    for (int s = 0; s < 3; ++s)
        CK(cudaMemcpyAsync(&c->d_ctl->n[s], &nn[s], sizeof(nn[s]), cudaMemcpyHostToDevice, c->stream));
    c->launch_t0.push_back(c->t);
    k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, c->sp[0].cap, c->sp[1].cap, c->sp[2].cap);
    CK(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
    if (c->learn_on) CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->d_heads, 0, 64 * sizeof(unsigned long long), c->stream));
    CK(cudaStreamSynchronize(c->stream));   // the host counts above are stack memory
    // pipeline: upload chunk i (copy stream) -> step chunk i (a launch over its
    // range with its own work counter, on two alternating compute streams, so
    // that the tail of one launch overlaps the next) -> download chunk i's
    // slots, updated in place (copy stream), unless the population is
    // compacted afterwards.  Launches of different chunks touch disjoint
    // slots; appends, spills and tallies are atomic.
    {
        const StepArgs A0 = make_args(c, dt, 1, 0, 0);
        CK(prepare_step(minb, smem, A0.general != 0, A0.event != 0, A0.learn != 0));
    }
    const long long G = n[0] + n[1] + n[2];
    const long long cs = std::max<long long>(1, (G + nchunks - 1) / nchunks);
    int nch = direct ? 0 : int((G + cs - 1) / cs);
    if (direct) {
        // one population launch over everything, reading the host slots and
        // writing results to the host arrays; the spill passes and the learned
        // round below append there too
        for (int s = 0; s < 3; ++s) {
            if (n[s] > 0) {
                c->hin_xw[s] = static_cast<const float4*>(hv[s][0]);
                c->hin_ps[s] = static_cast<const float4*>(hv[s][1]);
                c->hin_meta[s] = static_cast<const uint4*>(hv[s][2]);
            }
            if (out_cap[s] > 0) {
                c->hx_xw[s] = static_cast<float4*>(hv[s][3]);
                c->hx_ps[s] = static_cast<float4*>(hv[s][4]);
                c->hx_meta[s] = static_cast<uint4*>(hv[s][5]);
                c->hx_cap[s] = out_cap[s];
            }
        }
        StepArgs A = make_args(c, dt, 1, 0, 0);
        CK(cudaEventRecord(c->io_tev[0], c->stream));
        CK(launch_step_prepared(minb, grid_blocks(c), threads, smem, c->stream, A));
        CK(cudaEventRecord(c->io_tev[1], c->stream));
        c->launches += 1;
    }
    for (int i = 0; i < nch; ++i) {
        const long long g0 = i * cs, g1 = std::min(G, g0 + cs);
        long long a[3], b[3];
        chunk_ranges(n, g0, g1, a, b);
        cudaEvent_t up = c->io_ev[2 * i], done = c->io_ev[2 * i + 1];
        for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], in[s], a[s], b[s], true, c->s_h2d));
        CK(cudaEventRecord(up, c->s_h2d));
        cudaStream_t cs_i = (i & 1) ? c->s_cmp : c->stream;
        CK(cudaStreamWaitEvent(cs_i, up, 0));
        StepArgs A = make_args(c, dt, 1, 0, 0);
        A.g_lo = g0;
        A.g_hi = g1;
        A.head = c->d_heads + i;
        CK(cudaEventRecord(c->io_tev[2 * i], cs_i));
        CK(launch_step_prepared(minb, grid_blocks(c), threads, smem, cs_i, A));
        CK(cudaEventRecord(c->io_tev[2 * i + 1], cs_i));
        c->launches += 1;
        CK(cudaEventRecord(done, cs_i));
        if (!compact) {
            CK(cudaStreamWaitEvent(c->s_d2h, done, 0));
            for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], out[s], a[s], b[s], false, c->s_d2h));
        }
    }
    // both compute streams joined, then the spill passes and the learned
    // round, as in a launch group
    CK(cudaEventRecord(c->io_join, c->s_cmp));
    CK(cudaStreamWaitEvent(c->stream, c->io_join, 0));
    {
        StepArgs P0 = make_args(c, dt, 1, 1, 1), P1 = make_args(c, dt, 1, 1, 0);
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P0));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P1));
        c->launches += 4;
        if (c->learn_on) {
            CK(enqueue_learned_round(c, dt, 1, minb, threads, smem));
            CK(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
        }
        CK(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           c->stream));
        if ((rc = readback(c))) return rc;
        if (c->learn_on) count_learned(c);
        for (int i = 0; i < std::max(nch, direct ? 1 : 0); ++i) {   // step-kernel time of the launches
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, c->io_tev[2 * i], c->io_tev[2 * i + 1]));
            c->k_ms += ms;
            c->k_launches += 1;
        }
        unsigned long long pending = c->h_spn[1];
        bool host_passes = false;
        if ((rc = drain_spills(c, dt, 1, threads, smem, 1, -1, &host_passes, &pending))) return rc;
        if (host_passes && (rc = readback(c))) return rc;
    }
    if (c->h_ctl->timeout) return fail(c, PCL_ERR_TIMEOUT, "table staging wait timed out");
    c->t = tfinal;
    c->steps += 1;
    c->particle_steps += (long long)c->h_ctl->live_start[0];
    for (int s = 0; s < 3; ++s) c->live[s] = (long long)c->h_ctl->live_end[0][s];
    if (c->h_ctl->err[PCL_E_CAPACITY] > 0) return fail(c, PCL_ERR_CAPACITY, "population capacity exceeded");
    long long from[3] = {n[0], n[1], n[2]};   // slots the host arrays do not hold yet
    if (compact) {
        if ((rc = compact_all(c)) || (rc = readback(c))) return rc;
        for (int s = 0; s < 3; ++s) from[s] = 0;   // everything is downloaded below
    } else {
        c->steps_since_compact += 1;
    }
    // the rest: appended secondaries (or the whole compacted population); in
    // host-direct mode the kernels wrote the appended slots to the host already
    long long nf[3];
    for (int s = 0; s < 3; ++s) {
        nf[s] = (c->sp[s].set && c->sp[s].cap > 0) ? std::min<long long>((long long)c->h_ctl->n[s], c->sp[s].cap) : 0;
        if (nf[s] > out_cap[s]) return fail(c, PCL_ERR_CAPACITY, "output arrays too small");
        if (direct && !compact) from[s] = nf[s];
    }
    for (int s = 0; s < 3; ++s) CK(copy_slots(c->sp[s], out[s], from[s], nf[s], false, c->s_d2h));
    CK(cudaStreamSynchronize(c->s_d2h));
    for (int s = 0; s < 3; ++s) n_out[s] = nf[s];
    return PCL_OK;
}

int pcl_host_register(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return PCL_ERR_INVALID;
    return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

int pcl_host_unregister(void* ptr) {
    if (!ptr) return PCL_ERR_INVALID;
    return cudaHostUnregister(ptr) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

int pcl_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return PCL_ERR_INVALID;
    *ptr = nullptr;
    if (bytes == 0) return PCL_ERR_INVALID;
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return PCL_ERR_CUDA;
    *ptr = p;
    return PCL_OK;
}

int pcl_host_free(void* ptr) {
    if (!ptr) return PCL_ERR_INVALID;
    return cudaFreeHost(ptr) == cudaSuccess ? PCL_OK : PCL_ERR_CUDA;
}

}  // extern "C"
