// C ABI: learned samplers - attaching networks to table positions, training
// data from the table samplers, statistics, and the sampler test hook.
#include "ctx_internal.cuh"

using namespace pcl;

extern "C" {

static int learn_kind_ok(const pcl_process& P, int kind) {
    return (kind == PCL_LEARN_SB && P.kind == PCL_PROC_SELTZER_BERGER) ||
           (kind == PCL_LEARN_MOLLER && P.kind == PCL_PROC_MOLLER);
}

int pcl_set_learned(void* ctx, int species, int proc_index, int kind, void* mlp) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc || proc_index >= 16) return fail(c, PCL_ERR_INVALID, "process index");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (!mlp) {
        c->learn_net[species][proc_index] = nullptr;
        c->learn_kind[species][proc_index] = 0;
        c->learn_ok[species][proc_index][0] = c->learn_ok[species][proc_index][1] = 0u;
    } else {
        if (!learn_kind_ok(S.procs[proc_index], kind))
            return fail(c, PCL_ERR_UNSUPPORTED, "learned sampler kind does not match the process");
        // where the network is monotone in u: 64 bins of a, 4 energies each, 257 values of u
        const int nb = 64, ne = 4, nu = 257;
        std::vector<float> x(2 * nb * ne * nu), y(nb * ne * nu);
        for (int b = 0; b < nb; ++b)
            for (int e = 0; e < ne; ++e)
                for (int i = 0; i < nu; ++i) {
                    size_t r = (size_t(b) * ne + e) * nu + i;
                    x[2 * r] = -1.0f + (float(b) + (float(e) + 0.5f) / ne) * (2.0f / nb);
                    x[2 * r + 1] = 2.0f * (float(i) + 0.5f) / nu - 1.0f;
                }
        rc = pcl_mlp_forward(mlp, int64_t(y.size()), x.data(), y.data());
        if (rc) return fail(c, rc, std::string("network evaluation: ") + pcl_mlp_last_error(mlp));
        uint32_t ok[2] = {0u, 0u};
        for (int b = 0; b < nb; ++b) {
            bool mono = true;
            for (int e = 0; e < ne && mono; ++e)
                for (int i = 1; i < nu && mono; ++i) {
                    size_t r = (size_t(b) * ne + e) * nu + i;
                    if (!(y[r] >= y[r - 1]) || !std::isfinite(y[r])) mono = false;
                }
            if (mono) ok[b >> 5] |= 1u << (b & 31);
        }
        c->learn_net[species][proc_index] = mlp;
        c->learn_kind[species][proc_index] = kind;
        c->learn_ok[species][proc_index][0] = ok[0];
        c->learn_ok[species][proc_index][1] = ok[1];
    }
    // distinct networks and the pick table
    c->nets.clear();
    for (int k = 0; k < 48; ++k) c->pick.net[k] = -1;
    for (int sp = 0; sp < 3; ++sp)
        for (int j = 0; j < 16; ++j) {
            void* n = c->learn_net[sp][j];
            if (!n) continue;
            int idx = -1;
            for (size_t q = 0; q < c->nets.size(); ++q)
                if (c->nets[q] == n) idx = int(q);
            if (idx < 0) { idx = int(c->nets.size()); c->nets.push_back(n); }
            c->pick.net[sp * 16 + j] = int8_t(idx);
        }
    c->learn_on = !c->nets.empty();
    c->blob_dirty = true;
    return ensure_lq(c);
}

int pcl_time_energy_draw(void* ctx, int species, int proc_index, int kind, void* mlp, int64_t n, int reps,
                         double* ms_table, double* ms_net, float* out_table, float* out_net, uint32_t* draws_table) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc) return fail(c, PCL_ERR_INVALID, "process index");
    if (!mlp || n < 1 || n > (1ll << 26) || reps < 1 || reps > 100 || !ms_table || !ms_net)
        return fail(c, PCL_ERR_INVALID, "time_energy_draw arguments");
    if (!learn_kind_ok(S.procs[proc_index], kind))
        return fail(c, PCL_ERR_UNSUPPORTED, "learned sampler kind does not match the process");
    CK(cudaSetDevice(c->device));
    if ((rc = build_blob(c))) return rc;
    float *d_t = nullptr, *d_n = nullptr, *d_x = nullptr, *d_y = nullptr;
    uint32_t* d_draws = nullptr;
    unsigned long long* d_cnt = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    struct Free {
        float **a, **b, **x, **y; uint32_t** d; unsigned long long** cnt; cudaEvent_t *e0, *e1; cudaStream_t s;
        ~Free() {
            cudaStreamSynchronize(s);
            cudaFree(*a); cudaFree(*b); cudaFree(*x); cudaFree(*y); cudaFree(*d); cudaFree(*cnt);
            if (*e0) cudaEventDestroy(*e0);
            if (*e1) cudaEventDestroy(*e1);
        }
    } fr{&d_t, &d_n, &d_x, &d_y, &d_draws, &d_cnt, &e0, &e1, c->stream};
    CK(cudaMalloc(&d_t, sizeof(float) * n));
    CK(cudaMalloc(&d_n, sizeof(float) * n));
    CK(cudaMalloc(&d_x, sizeof(float) * 2 * n));
    CK(cudaMalloc(&d_y, sizeof(float) * n));
    CK(cudaMalloc(&d_draws, sizeof(uint32_t) * n));
    CK(cudaMalloc(&d_cnt, sizeof(unsigned long long)));
    const unsigned long long nn = (unsigned long long)n;
    CK(cudaMemcpy(d_cnt, &nn, sizeof(nn), cudaMemcpyHostToDevice));
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    StepArgs A = make_args(c, 0.0, 1, 0, 0);
    const size_t smem = c->blob.size() + 16;
    CK(cudaFuncSetAttribute(k_draw_table, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    CK(cudaFuncSetAttribute(k_draw_net_map, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int grid = int(std::max<long long>(1, std::min<long long>((n + 255) / 256, 8ll * c->sm_count)));
    const unsigned long long sid_t = 0xB1ull << 56, sid_n = 0xB2ull << 56;
    double bt = 1e30, bn = 1e30;
    for (int r = 0; r < reps; ++r) {
        float ms = 0.0f;
        CK(cudaEventRecord(e0, c->stream));
        k_draw_table<<<grid, 256, smem, c->stream>>>(A, species, proc_index, kind, n, sid_t, d_t, d_draws);
        CK(cudaGetLastError());
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        bt = std::min(bt, double(ms));
        CK(cudaEventRecord(e0, c->stream));
        k_draw_net_x<<<grid, 256, 0, c->stream>>>(n, sid_n, A.key0, A.key1, d_x);
        CK(cudaGetLastError());
        CK(mlp::infer_multi(&mlp, 1, d_x, d_cnt, n, d_y, n, c->stream));
        k_draw_net_map<<<grid, 256, smem, c->stream>>>(A, species, proc_index, kind, n, d_y, d_n);
        CK(cudaGetLastError());
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        bn = std::min(bn, double(ms));
    }
    if (out_table) CK(cudaMemcpy(out_table, d_t, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (out_net) CK(cudaMemcpy(out_net, d_n, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (draws_table) CK(cudaMemcpy(draws_table, d_draws, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    *ms_table = bt;
    *ms_net = bn;
    // a network whose tensor-core wait gave up flags its handle; report it here
    float probe[2] = {0.0f, 0.0f}, py = 0.0f;
    if (pcl_mlp_forward(mlp, 1, probe, &py) == PCL_ERR_TIMEOUT)
        return fail(c, PCL_ERR_TIMEOUT, "network inference timed out");
    return PCL_OK;
}

int pcl_learn_data(void* ctx, int species, int proc_index, int kind, int nT, int64_t per_T, int Q, uint64_t seed,
                   float* x_out, float* t_out, int64_t* nrows) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc) return fail(c, PCL_ERR_INVALID, "process index");
    if (nT < 2 || nT > 65536 || per_T < 1 || Q < 2 || !x_out || !t_out || !nrows)
        return fail(c, PCL_ERR_INVALID, "learn_data sizes");
    const pcl_process& P = S.procs[proc_index];
    if (!learn_kind_ok(P, kind)) return fail(c, PCL_ERR_UNSUPPORTED, "learned sampler kind does not match the process");
    CK(cudaSetDevice(c->device));
    if ((rc = build_blob(c))) return rc;
    const int nbins = 4096;
    const float hmin = 0.0f, hmax = 1.0f;   // both output variables lie in [0, 1]
    unsigned int* hist = nullptr;
    const size_t hn = size_t(nT) * nbins;
    CK(cudaMallocAsync(&hist, sizeof(unsigned int) * hn, c->stream));
    CK(cudaMemsetAsync(hist, 0, sizeof(unsigned int) * hn, c->stream));
    StepArgs A = make_args(c, 0.0, 1, 0, 0);
    const size_t smem = c->blob.size() + 16;
    CK(cudaFuncSetAttribute(k_learn_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const long long total = (long long)nT * per_T;
    const int grid = int(std::max<long long>(1, std::min<long long>((total + 255) / 256, 8ll * c->sm_count)));
    const unsigned long long sid_base = (0xA5ull << 56) | ((seed & 0xFFFFull) << 40);
    k_learn_hist<<<grid, 256, smem, c->stream>>>(A, species, proc_index, kind, nT, (long long)per_T, nbins, hmin, hmax,
                                                  sid_base, hist);
    CK(cudaGetLastError());
    std::vector<unsigned int> h(hn);
    CK(cudaMemcpyAsync(h.data(), hist, sizeof(unsigned int) * hn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaFreeAsync(hist, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const double dh = double(hmax - hmin) / nbins;
    int64_t r = 0;
    std::vector<double> cum(nbins + 1);
    for (int g = 0; g < nT; ++g) {
        const double a = -1.0 + 2.0 * g / double(nT - 1);
        if (kind == PCL_LEARN_MOLLER) {
            const double T = std::pow(10.0, 6.0 + 2.0 * a) * si::e;
            if (!(P.param[0] < 0.45 * T)) continue;   // degenerate kinematic range: no rows
        }
        const unsigned int* hg = h.data() + size_t(g) * nbins;
        cum[0] = 0.0;
        for (int b = 0; b < nbins; ++b) cum[b + 1] = cum[b] + hg[b];
        const double N = cum[nbins];
        if (N <= 0) continue;
        int b = 0;
        for (int i = 0; i < Q; ++i) {
            const double u = (i + 0.5) / Q;
            const double target = u * N;
            while (b < nbins - 1 && cum[b + 1] < target) ++b;
            const double f = hg[b] ? (target - cum[b]) / hg[b] : 0.5;
            x_out[2 * r] = float(a);
            x_out[2 * r + 1] = float(2.0 * u - 1.0);
            t_out[r] = float(hmin + (b + std::min(1.0, std::max(0.0, f))) * dh);
            ++r;
        }
    }
    *nrows = r;
    return PCL_OK;
}

int pcl_learn_stats(void* ctx, int64_t* suspended, int64_t* rounds) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (suspended) *suspended = c->learn_suspended;
    if (rounds) *rounds = c->learn_rounds;
    return PCL_OK;
}

int pcl_test_sampler(void* ctx, int species, int proc_index, int64_t n, const double* p, const uint64_t* sid,
                     double* out_p, double* out_s, int32_t* out_kind, uint32_t* out_ctr) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (proc_index < 0 || proc_index >= S.nproc) return fail(c, PCL_ERR_INVALID, "process index");
    if (n <= 0 || !p || !sid || !out_p || !out_s || !out_kind || !out_ctr) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    if ((rc = build_blob(c))) return rc;
    std::vector<float> hp(3 * n);
    std::vector<uint32_t> hs(2 * n);
    for (int64_t i = 0; i < 3 * n; ++i) hp[i] = float(p_to_dev(p[i]));
    for (int64_t i = 0; i < n; ++i) { hs[2 * i] = uint32_t(sid[i]); hs[2 * i + 1] = uint32_t(sid[i] >> 32); }
    float *dp = nullptr, *dop = nullptr, *dos = nullptr;
    uint32_t *dsid = nullptr, *dctr = nullptr;
    int* dkind = nullptr;
    CK(cudaMalloc(&dp, sizeof(float) * 3 * n));
    CK(cudaMalloc(&dsid, sizeof(uint32_t) * 2 * n));
    CK(cudaMalloc(&dop, sizeof(float) * 9 * n));
    CK(cudaMalloc(&dos, sizeof(float) * 3 * n));
    CK(cudaMalloc(&dkind, sizeof(int) * 3 * n));
    CK(cudaMalloc(&dctr, sizeof(uint32_t) * n));
    CK(h2d(c, dp, hp.data(), sizeof(float) * 3 * n));
    CK(h2d(c, dsid, hs.data(), sizeof(uint32_t) * 2 * n));
    CK(cudaMemsetAsync(dop, 0, sizeof(float) * 9 * n, c->stream));
    CK(cudaMemsetAsync(dos, 0, sizeof(float) * 3 * n, c->stream));
    StepArgs A = make_args(c, 0.0, 1, 0, 0);
    size_t smem = c->blob.size() + 16;
    CK(cudaFuncSetAttribute(k_test_sampler, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int blocks = int((n + 127) / 128);
    k_test_sampler<<<blocks, 128, smem, c->stream>>>(A, species, proc_index, n, dp, dsid, dop, dos, dkind, dctr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    std::vector<float> hop(9 * n), hos(3 * n);
    CK(d2h(c, hop.data(), dop, sizeof(float) * 9 * n));
    CK(d2h(c, hos.data(), dos, sizeof(float) * 3 * n));
    CK(d2h(c, out_kind, dkind, sizeof(int) * 3 * n));
    CK(d2h(c, out_ctr, dctr, sizeof(uint32_t) * n));
    for (int64_t i = 0; i < 9 * n; ++i) out_p[i] = p_to_si(hop[i]);
    for (int64_t i = 0; i < 3 * n; ++i) out_s[i] = hos[i];
    cudaFree(dp); cudaFree(dsid); cudaFree(dop); cudaFree(dos); cudaFree(dkind); cudaFree(dctr);
    return PCL_OK;
}

}  // extern "C"
