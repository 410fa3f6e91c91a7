// C ABI: population operations - roulette! / split! (whole population and per
// swarm), the device population cap, WallCallback records, batched-swarm
// setup and statistics, energy spectra.
#include "ctx_internal.cuh"

using namespace pcl;

extern "C" {

int pcl_roulette(void* ctx, int species, double pkeep) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (!(pkeep > 0.0 && pkeep <= 1.0)) return fail(c, PCL_ERR_INVALID, "keep probability must be in (0, 1]");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    // the removed count in the context's reusable scratch (no allocation per call)
    if ((rc = ensure_scratch(c, 256))) return rc;
    unsigned long long* killed = static_cast<unsigned long long*>(c->d_scr);
    CK(cudaMemsetAsync(killed, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    k_roulette<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], n, float(pkeep), uint32_t(c->cfg.seed),
                                            uint32_t(c->cfg.seed >> 32), killed);
    CK(cudaGetLastError());
    unsigned long long hk = 0;
    CK(cudaMemcpyAsync(&hk, killed, sizeof(hk), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = std::max<long long>(0, c->live[species] - (long long)hk);
    return PCL_OK;
}

int pcl_roulette_swarms(void* ctx, int species, int nswarm, const double* pkeep) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !pkeep || nswarm < 1 || nswarm > 256) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    std::vector<float> q(nswarm);
    for (int i = 0; i < nswarm; ++i) {
        if (!(pkeep[i] > 0.0)) return fail(c, PCL_ERR_INVALID, "keep probabilities must be > 0");
        q[i] = float(std::min(1.0, pkeep[i]));
    }
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    if ((rc = ensure_scratch(c, 256 + sizeof(float) * nswarm))) return rc;
    unsigned long long* killed = static_cast<unsigned long long*>(c->d_scr);
    float* dq = reinterpret_cast<float*>(static_cast<char*>(c->d_scr) + 256);
    CK(cudaMemcpyAsync(dq, q.data(), sizeof(float) * nswarm, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(killed, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    k_roulette_swarms<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], n, dq, nswarm,
                                                   uint32_t(c->cfg.seed), uint32_t(c->cfg.seed >> 32), killed);
    CK(cudaGetLastError());
    unsigned long long hk = 0;
    CK(cudaMemcpyAsync(&hk, killed, sizeof(hk), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = std::max<long long>(0, c->live[species] - (long long)hk);
    return PCL_OK;
}

int pcl_split(void* ctx, int species, double p) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (!(p >= 0.0 && p <= 64.0)) return fail(c, PCL_ERR_INVALID, "mean number of copies must be in [0, 64]");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long n = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, n)) || n == 0) return rc;
    // the lost count in the context's reusable scratch (no allocation per call)
    if ((rc = ensure_scratch(c, 256))) return rc;
    unsigned long long* lost = static_cast<unsigned long long*>(c->d_scr);
    CK(cudaMemsetAsync(lost, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((n + 255) / 256, 8ll * c->sm_count));
    const float pf = float(p);
    k_split<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], n, S.cap, pf,
                                         std::exp(-double(pf)), c->nswarm, uint32_t(c->cfg.seed),
                                         uint32_t(c->cfg.seed >> 32), &c->d_ctl->n[species], lost);
    CK(cudaGetLastError());
    unsigned long long hl = 0;
    CK(cudaMemcpyAsync(&hl, lost, sizeof(hl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    long long nn = 0;
    if ((rc = get_n(c, species, nn))) return rc;
    c->live[species] += nn - n;
    if (hl) return fail(c, PCL_ERR_CAPACITY, "split copies beyond the population capacity were lost");
    return PCL_OK;
}

// A table of f(E) for pcl_roulette_fn / pcl_split_fn: 1 to 4096 nodes, the
// energies (J) finite, >= 0 and strictly increasing, the values finite and
// within [vmin, vmax]; copied to the context's scratch (after its first 256 B)
// as the device evaluates it (table_fn): the energies in units of m_e c^2,
// the values, the slopes of the intervals, the energies rounded to FP32.
static int stage_table(Ctx* c, int n, const double* energy, const double* value, double vmin, double vmax,
                       const double** dtab) {
    if (n < 1 || n > 4096 || !energy || !value) return fail(c, PCL_ERR_INVALID, "table of 1 to 4096 nodes");
    const size_t nd = 3 * size_t(n) + (size_t(n) + 1) / 2;
    std::vector<double> h(nd, 0.0);
    for (int i = 0; i < n; ++i) {
        if (!std::isfinite(energy[i]) || energy[i] < 0.0 || (i > 0 && !(energy[i] > energy[i - 1])))
            return fail(c, PCL_ERR_INVALID, "table energies must be finite, >= 0 and strictly increasing");
        if (!std::isfinite(value[i]) || value[i] < vmin || value[i] > vmax)
            return fail(c, PCL_ERR_INVALID, "table value out of range");
        h[i] = energy[i] / si::mc2;
        h[n + i] = value[i];
    }
    for (int i = 0; i + 1 < n; ++i) {
        h[2 * n + i] = (h[n + i + 1] - h[n + i]) / (h[i + 1] - h[i]);
        if (!std::isfinite(h[2 * n + i])) return fail(c, PCL_ERR_INVALID, "table nodes too close");
    }
    float* f = reinterpret_cast<float*>(h.data() + 3 * size_t(n));
    for (int i = 0; i < n; ++i) f[i] = float(h[i]);
    int rc = ensure_scratch(c, 256 + sizeof(double) * nd);
    if (rc) return rc;
    double* d = reinterpret_cast<double*>(static_cast<char*>(c->d_scr) + 256);
    CK(cudaMemcpyAsync(d, h.data(), sizeof(double) * nd, cudaMemcpyHostToDevice, c->stream));
    *dtab = d;
    return PCL_OK;
}

int pcl_roulette_fn(void* ctx, int species, int n, const double* energy, const double* pkeep) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long np = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, np)) || np == 0) return rc;
    const double* dtab = nullptr;
    if ((rc = stage_table(c, n, energy, pkeep, -1e300, 1e300, &dtab))) return rc;
    unsigned long long* killed = static_cast<unsigned long long*>(c->d_scr);
    CK(cudaMemsetAsync(killed, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((np + 255) / 256, 8ll * c->sm_count));
    k_roulette_fn<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], np, species, dtab, n,
                                               uint32_t(c->cfg.seed), uint32_t(c->cfg.seed >> 32), killed);
    CK(cudaGetLastError());
    unsigned long long hk = 0;
    CK(cudaMemcpyAsync(&hk, killed, sizeof(hk), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->live[species] = std::max<long long>(0, c->live[species] - (long long)hk);
    return PCL_OK;
}

int pcl_split_fn(void* ctx, int species, int n, const double* energy, const double* mean) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    long long np = 0;
    if (S.cap <= 0 || (rc = get_n(c, species, np)) || np == 0) return rc;
    const double* dtab = nullptr;
    if ((rc = stage_table(c, n, energy, mean, 0.0, 64.0, &dtab))) return rc;
    unsigned long long* lost = static_cast<unsigned long long*>(c->d_scr);
    CK(cudaMemsetAsync(lost, 0, sizeof(unsigned long long), c->stream));
    const int grid = int(std::min<long long>((np + 255) / 256, 8ll * c->sm_count));
    k_split_fn<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], np, S.cap, species, dtab, n,
                                            c->nswarm, uint32_t(c->cfg.seed), uint32_t(c->cfg.seed >> 32),
                                            &c->d_ctl->n[species], lost);
    CK(cudaGetLastError());
    unsigned long long hl = 0;
    CK(cudaMemcpyAsync(&hl, lost, sizeof(hl), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    long long nn = 0;
    if ((rc = get_n(c, species, nn))) return rc;
    c->live[species] += nn - np;
    if (hl) return fail(c, PCL_ERR_CAPACITY, "split copies beyond the population capacity were lost");
    return PCL_OK;
}

int pcl_set_wall(void* ctx, int species, int coord, double v, int drop, int64_t capacity) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (coord < -1 || coord > 2 || capacity < 0 || capacity > (1ll << 30))
        return fail(c, PCL_ERR_INVALID, "wall axis or capacity");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    SpeciesState& S = c->sp[species];
    S.wall_coord = coord;
    S.wall_v = v;
    S.wall_drop = drop ? 1 : 0;
    if (coord >= 0 && capacity > c->wall_cap) {
        cudaFree(c->d_wall_xw); cudaFree(c->d_wall_pt); cudaFree(c->d_wall_meta); cudaFree(c->d_wall_n);
        c->d_wall_xw = c->d_wall_pt = nullptr; c->d_wall_meta = nullptr; c->d_wall_n = nullptr; c->wall_cap = 0;
        CK(cudaMalloc(&c->d_wall_xw, sizeof(float4) * capacity));
        CK(cudaMalloc(&c->d_wall_pt, sizeof(float4) * capacity));
        CK(cudaMalloc(&c->d_wall_meta, sizeof(uint4) * capacity));
        CK(cudaMalloc(&c->d_wall_n, sizeof(unsigned long long)));
        CK(cudaMemset(c->d_wall_n, 0, sizeof(unsigned long long)));
        c->wall_cap = capacity;
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_get_wall(void* ctx, int64_t* n, int32_t* species, uint64_t* sid, double* x, double* p, double* w, double* t) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !n) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    if (!c->d_wall_n) { *n = 0; return PCL_OK; }
    unsigned long long cnt = 0;
    CK(d2h(c, &cnt, c->d_wall_n, sizeof(cnt)));
    const long long m = std::min<long long>((long long)cnt, c->wall_cap);
    if (!species) { *n = m; return PCL_OK; }   // query
    if (*n < m) { *n = m; return fail(c, PCL_ERR_INVALID, "output arrays too short for the wall records"); }
    std::vector<float4> xw(m), pt(m);
    std::vector<uint4> meta(m);
    if (m > 0) {
        CK(d2h(c, xw.data(), c->d_wall_xw, sizeof(float4) * m));
        CK(d2h(c, pt.data(), c->d_wall_pt, sizeof(float4) * m));
        CK(d2h(c, meta.data(), c->d_wall_meta, sizeof(uint4) * m));
    }
    for (long long i = 0; i < m; ++i) {
        species[i] = int32_t(meta[i].z);
        sid[i] = uint64_t(meta[i].x) | (uint64_t(meta[i].y) << 32);
        x[3 * i] = xw[i].x; x[3 * i + 1] = xw[i].y; x[3 * i + 2] = xw[i].z;
        w[i] = xw[i].w;
        p[3 * i] = p_to_si(pt[i].x); p[3 * i + 1] = p_to_si(pt[i].y); p[3 * i + 2] = p_to_si(pt[i].z);
        const size_t li = std::min<size_t>(meta[i].w, c->launch_t0.size() - 1);
        t[i] = c->launch_t0[li] + double(pt[i].w) * NS;
    }
    *n = m;
    const unsigned long long zero = 0;
    CK(h2d(c, c->d_wall_n, &zero, sizeof(zero)));
    return (long long)cnt > c->wall_cap ? fail(c, PCL_ERR_CAPACITY, "wall records beyond capacity were lost")
                                         : PCL_OK;
}

int pcl_set_swarms(void* ctx, int nswarm, const double* E, const double* Fdt, double safety) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (nswarm < 0 || nswarm > 256 || (nswarm > 0 && (!E || !Fdt)) || !(safety >= 0))
        return fail(c, PCL_ERR_INVALID, "bad swarm description");
    c->nswarm = nswarm;
    c->swarm_safety = safety;
    if (nswarm > 0) {
        c->swarm_E.assign(E, E + 3 * size_t(nswarm));
        c->swarm_Fdt.assign(Fdt, Fdt + nswarm);
    } else {
        c->swarm_E.clear();
        c->swarm_Fdt.clear();
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_swarm_moments(void* ctx, int species, int nswarm, double* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nswarm < 1 || nswarm > 256) return fail(c, PCL_ERR_INVALID, "nswarm out of range");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    const int len = 6 * nswarm;
    const int blocks = int(std::max<long long>(1, std::min<long long>(2ll * c->sm_count, (slots + 255) / 256)));
    if ((rc = ensure_scratch(c, sizeof(double) * len * (blocks + 1)))) return rc;
    double* d = static_cast<double*>(c->d_scr);
    double* part = d + len;
    if (slots > 0) {
        k_swarm_moments<<<blocks, 256, sizeof(double) * len, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur],
                                                                          slots, species, nswarm, part);
        CK(cudaGetLastError());
    } else {
        CK(cudaMemsetAsync(part, 0, sizeof(double) * len * blocks, c->stream));
    }
    k_swarm_reduce<<<(len + 7) / 8, 256, 0, c->stream>>>(part, blocks, len, d);   // one warp per value
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d, sizeof(double) * len, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < nswarm; ++k) out[6 * k + 2] = e_to_si(out[6 * k + 2]);
    return PCL_OK;
}

int pcl_energy_histogram(void* ctx, int species, int swarm, int nedges, const double* edges, int64_t* counts,
                         double* weights) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !edges || !counts || !weights) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nedges < 2 || nedges > PCL_MAX_HIST_EDGES) return fail(c, PCL_ERR_INVALID, "nedges out of range");
    if (swarm < -1 || swarm >= std::max(1, c->nswarm) || (swarm >= 0 && c->nswarm == 0))
        return fail(c, PCL_ERR_INVALID, "swarm out of range");
    std::vector<double> ed(nedges);
    for (int i = 0; i < nedges; ++i) {
        if (!(std::isfinite(edges[i]) && edges[i] >= 0.0) || (i > 0 && !(edges[i] > edges[i - 1])))
            return fail(c, PCL_ERR_INVALID, "edges must be finite, >= 0 and strictly increasing");
        ed[i] = e_to_dev(edges[i]);
    }
    const int nb = nedges - 1;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    std::vector<unsigned long long> hc(nb, 0ull);
    std::vector<double> hw(nb, 0.0);
    if (S.cap > 0) {
        // scratch: counts [nb] (u64), weights [nb], edges [nb + 1]
        if ((rc = ensure_scratch(c, sizeof(double) * (3 * size_t(nb) + 1)))) return rc;
        unsigned long long* dc = static_cast<unsigned long long*>(c->d_scr);
        double* dw = reinterpret_cast<double*>(dc + nb);
        double* de = dw + nb;
        CK(cudaMemcpyAsync(de, ed.data(), sizeof(double) * nedges, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemsetAsync(dc, 0, 2 * sizeof(double) * nb, c->stream));
        // shared: edges [nb + 1] and weights [nb] (FP64), counts and weight-1 counts [nb] (u32),
        // FP32 edges [nb + 1]
        const size_t smem = sizeof(double) * (2 * size_t(nb) + 1) + 2 * sizeof(unsigned int) * nb +
                            sizeof(float) * (size_t(nb) + 1);
        CK(cudaFuncSetAttribute(k_energy_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(sizeof(double) * (2 * PCL_MAX_HIST_EDGES) + 12 * PCL_MAX_HIST_EDGES)));
        const long long bps = std::max<long long>(1, std::min<long long>(8, (200ll << 10) / (long long)smem));
        const int grid = int(std::min<long long>((S.cap + 255) / 256, bps * c->sm_count));
        k_energy_hist<<<grid, 256, smem, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], &c->d_ctl->n[species],
                                                      S.cap, species, swarm, de, nb, dc, dw);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(hc.data(), dc, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(hw.data(), dw, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    for (int i = 0; i < nb; ++i) {
        counts[i] = (int64_t)hc[i];
        weights[i] = hw[i];
    }
    return PCL_OK;
}

int pcl_swarm_counts(void* ctx, int species, int nswarm, int64_t* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nswarm < 1 || nswarm > 256) return fail(c, PCL_ERR_INVALID, "nswarm out of range");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    std::vector<unsigned int> h(nswarm, 0u);
    if (S.cap > 0) {
        unsigned int* cnt = c->d_swcnt + 256 * species;
        const int grid = int(std::min<long long>((S.cap + 255) / 256, 4ll * c->sm_count));
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned int) * nswarm, c->stream));
        k_swarm_count<<<grid, 256, 0, c->stream>>>(S.meta[S.cur], &c->d_ctl->n[species], S.cap, nswarm, cnt);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(h.data(), cnt, sizeof(unsigned int) * nswarm, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    for (int k = 0; k < nswarm; ++k) out[k] = (int64_t)h[k];
    return PCL_OK;
}

int pcl_set_swarm_cap(void* ctx, int species, int64_t cap) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (cap < 0 || cap > (int64_t)0xffffffffll) return fail(c, PCL_ERR_INVALID, "cap out of range");
    c->swarm_cap[species] = (long long)cap;
    return PCL_OK;
}

}  // extern "C"
