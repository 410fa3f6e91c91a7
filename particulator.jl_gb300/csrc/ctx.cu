// Host side of the C ABI: the context, device memory, table packing, the step
// driver (advance! / run!), tallies, statistics and the launch-shape calls.
// Every entry point returns a PCL_* status and records a message for
// pcl_last_error.  Population operations, host I/O and the learned samplers
// live in ctx_popops.cu, ctx_hostio.cu and ctx_learn.cu.
#include "ctx_internal.cuh"

namespace pcl {

PCL_INTERNAL void free_species_buffers(SpeciesState& s) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(s.xw[b]); cudaFree(s.ps[b]); cudaFree(s.meta[b]);
        s.xw[b] = nullptr; s.ps[b] = nullptr; s.meta[b] = nullptr;
    }
    cudaFree(s.hist_n); cudaFree(s.hist_w);
    s.hist_n = nullptr; s.hist_w = nullptr;
}

PCL_INTERNAL int ensure_tiles(Ctx* c) {
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long nt = (capmax + kTile - 1) / kTile;
    if (nt < 1) nt = 1;
    if (nt <= c->tiles_cap) return PCL_OK;
    cudaFree(c->d_tile_cnt); cudaFree(c->d_tile_off);
    CK(cudaMalloc(&c->d_tile_cnt, sizeof(unsigned int) * 3 * nt));
    CK(cudaMalloc(&c->d_tile_off, sizeof(unsigned long long) * 3 * nt));
    c->tiles_cap = nt;
    return PCL_OK;
}

PCL_INTERNAL int ensure_spill(Ctx* c) {
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long want = std::max<long long>(1 << 16, capmax / 16);
    if (want <= c->sp_cap) return PCL_OK;
    for (int b = 0; b < 2; ++b) {
        cudaFree(c->sp_xw[b]); cudaFree(c->sp_ps[b]); cudaFree(c->sp_meta[b]);
        CK(cudaMalloc(&c->sp_xw[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->sp_ps[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->sp_meta[b], sizeof(uint4) * want));
    }
    c->sp_cap = want;
    return PCL_OK;
}

// ------------------------------------------------------------ blob pack --
static void pack_proc(const pcl_process& P, int sbi, DevProc& D) {
    std::memset(&D, 0, sizeof(D));
    D.kind = P.kind;
    D.sb = -1;
    using namespace si;
    switch (P.kind) {
        case PCL_PROC_MOLLER:
        case PCL_PROC_BHABHA:
            D.p[0] = float(P.param[0] / mc2);
            break;
        case PCL_PROC_RBEB:
            D.p[0] = float(P.param[0] / mc2);
            D.p[1] = float(P.param[1] / mc2);
            D.p[2] = float(P.param[2]);
            break;
        case PCL_PROC_REL_COULOMB: {
            double Z = (P.Z == 0) ? P.param[0] : double(P.Z);
            double a = 1.3413 * std::pow(Z, -1.0 / 3.0) * a_0;     // relativistic_coulomb.jl:14
            double lam = hbar / (m_e * c * a);
            D.p[0] = float(lam * lam / 4.0);                       // alpha = p[0] / p^2
            break;
        }
        case PCL_PROC_SELTZER_BERGER:
            D.sb = sbi;
            D.p[0] = float(P.Z);
            break;
        case PCL_PROC_PHOTOELECTRIC:
            D.nbind = std::min(P.nparam, 8);
            for (int m = 0; m < D.nbind; ++m) D.p[m] = float(P.param[m] / mc2);
            break;
        case PCL_PROC_BETHE_HEITLER: {
            double Z = P.Z;
            double aZ = alpha, aZ2 = aZ * aZ, aZ4 = aZ2 * aZ2, aZ6 = aZ4 * aZ2;  // _fc (bethe_heitler.jl:153-161)
            double fc = (1 / (1 + aZ2) + 0.20206 - 0.0369 * aZ2 + 0.0083 * aZ4 - 0.0020 * aZ6) * aZ2;
            double FZ = 8 * std::log(Z) / 3;
            D.p[0] = float(Z);
            D.p[1] = float(std::pow(Z, 1.0 / 3.0));
            D.p[2] = float(FZ);
            D.p[3] = float(FZ + 8 * fc);
            D.p[4] = float(2e6 * eV / mc2);
            D.p[5] = float(50e6 * eV / mc2);
            break;
        }
        case PCL_PROC_ELASTIC:
            D.p[0] = float(P.param[0]);
            break;
        case PCL_PROC_EXCITATION:
        case PCL_PROC_IONIZATION:
        case PCL_PROC_ATTACHMENT:
            D.p[0] = float(P.param[0] / mc2);
            break;
        default:
            break;
    }
}

PCL_INTERNAL int build_blob(Ctx* c) {
    if (!c->blob_dirty) return PCL_OK;
    using si::mc2;
    using si::e;
    using si::m_e;
    std::vector<float> data;
    auto off = [&]() { return int((sizeof(BlobHdr) / 4) + data.size()); };
    BlobHdr H;
    std::memset(&H, 0, sizeof(H));
    const float charge[3] = {-1.0f, 0.0f, 1.0f};
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        SpeciesHdr& h = H.sp[s];
        h.nproc = S.nproc;
        h.order = S.order;
        h.k = S.nint;
        h.tally_only = (S.flags & PCL_SPECIES_TALLY_ONLY) ? 1 : 0;
        h.xscale = float(1.0 / (S.xmax / mc2));
        h.cut = S.set ? float(S.cut / mc2) : INFINITY;
        h.charge = ((c->field_mask >> s) & 1) ? charge[s] : 0.0f;   // RestrictedForcing of the field
        h.frozen = ((c->push_mask >> s) & 1) ? 0 : 1;
        h.table_kind = S.table_kind;
        h.wall_coord = (S.wall_coord >= 0 && c->wall_cap > 0) ? S.wall_coord : -1;
        h.wall_v = float(S.wall_v);
        h.wall_drop = S.wall_drop;
        if (S.table_kind == 1) {
            h.lin_n = S.lin_n;
            h.lin_e0 = float(S.lin_e0 / mc2);
            h.lin_inv_step = float(1.0 / ((S.lin_e1 - S.lin_e0) / (S.lin_n - 1) / mc2));
            h.rate_off = off();
            for (size_t q = 0; q < S.rate.size(); ++q) data.push_back(float(rate_to_dev(S.rate[q])));
            h.rb_off = off();
            for (int i = 0; i < S.lin_n; ++i) data.push_back(float(rate_to_dev(S.rb[i])));
        } else {
            const int nI = S.nint + 1;
            h.rate_off = off();
            for (int i = 0; i < nI; ++i)
                for (int j = 0; j < S.nproc; ++j)
                    for (int k = 0; k < S.order; ++k)
                        data.push_back(float(rate_to_dev(S.rate[k + S.order * (j + S.nproc * i)])));
            h.rb_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k)
                    data.push_back(S.rb.empty() ? 0.0f : float(rate_to_dev(S.rb[k + S.order * i])));
        }
        h.cl_off = -1;
        if (c->cl_order > 0 && s != PCL_PHOTON && ((c->loss_mask >> s) & 1)) {
            const std::vector<double>& cf = (s == PCL_ELECTRON) ? c->cl_ec : c->cl_pc;
            h.cl_off = off();
            h.cl_k = c->cl_k;
            h.cl_order = c->cl_order;
            h.cl_xscale = float(1.0 / (c->cl_xmax / mc2));
            for (int i = 0; i <= c->cl_k; ++i)
                for (int k = 0; k < c->cl_order; ++k) data.push_back(float(force_to_dev(cf[k + c->cl_order * i])));
        }
        h.rbB_off = -1;
        if (c->nswarm > 0 && S.table_kind == 0 && S.nproc > 0 && s != PCL_PHOTON) {
            // swarm mode: the rate bound of swarm k is A + Fdt_k B (compratebound is linear in Fdt)
            const int nI = S.nint + 1;
            std::vector<double> A(size_t(S.order) * nI), Bt(size_t(S.order) * nI);
            pcl_ratebound_split(s, S.order, S.nproc, S.nint, S.xmax, S.rate.data(), c->swarm_safety, A.data(),
                                Bt.data());
            h.rb_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k) data.push_back(float(rate_to_dev(A[k + S.order * i])));
            h.rbB_off = off();
            for (int i = 0; i < nI; ++i)
                for (int k = 0; k < S.order; ++k) data.push_back(float(rate_to_dev(Bt[k + S.order * i])));
        }
        for (int j = 0; j < S.nproc; ++j) {
            pack_proc(S.procs[j], S.sb_index[j], h.proc[j]);
            h.proc[j].learn = c->learn_net[s][j] ? c->learn_kind[s][j] : 0;
            h.proc[j].learn_ok[0] = c->learn_ok[s][j][0];
            h.proc[j].learn_ok[1] = c->learn_ok[s][j][1];
        }
        if (S.hist_bins > 0) {
            h.hist_bins = S.hist_bins;
            double lmin = std::log(S.hist_emin / mc2), lmax = std::log(S.hist_emax / mc2);
            h.hist_lmin = float(lmin);
            h.hist_linv = float(S.hist_bins / (lmax - lmin));
        }
    }
    H.nsb = int(c->sb.size());
    for (size_t b = 0; b < c->sb.size(); ++b) {
        SBHdr& h = H.sb[b];
        h.ne = c->sb[b].ne;
        h.ncum = c->sb[b].ncum;
        h.inv_dp = float(c->sb[b].ncum - 1);
        double ym = 0.0;
        for (int j = 0; j + 1 < h.ne; ++j)
            ym = std::max(ym, std::fabs(c->sb[b].data[size_t(j + 1) * h.ncum] - c->sb[b].data[size_t(j) * h.ncum]));
        h.ymargin = float(ym);
        h.le_off = off();
        for (int j = 0; j < h.ne; ++j) data.push_back(float(c->sb[b].log_energy[j] - std::log(mc2)));
    }
    for (int a = 0; a < 3; ++a) {
        H.E[a] = float(force_to_dev(e * c->E[a]));            // per unit charge
        H.B[a] = float(e * c->B[a] / m_e * NS);
    }
    H.field_kind = c->field_kind;
    {
        const double* q = c->field_p;
        auto fe = [&](double v) { return float(force_to_dev(e * v)); };
        switch (c->field_kind) {
            case 1: H.fp[0] = float(q[0]); H.fp[1] = float(q[1]);
                    for (int a = 0; a < 3; ++a) H.fp[2 + a] = fe(q[2 + a]);
                    break;
            case 2: H.fp[0] = float(q[0]);
                    for (int a = 0; a < 6; ++a) H.fp[1 + a] = fe(q[1 + a]);
                    break;
            case 3: for (int a = 0; a < 3; ++a) {   // the widths as the reciprocals the device multiplies by
                        H.fp[a] = float(0.5 / (q[a] * q[a]));
                        H.fp[4 + a] = float(1.0 / (q[a] * q[a]));
                    }
                    H.fp[3] = fe(q[3]);
                    break;
            default: break;
        }
    }
    H.bfield_kind = c->bfield_kind;
    {
        const double* q = c->bfield_p;
        auto fb = [&](double v) { return float(e * v / m_e * NS); };
        switch (c->bfield_kind) {
            case 1: H.bp[0] = float(q[0]); H.bp[1] = float(q[1]);
                    for (int a = 0; a < 3; ++a) H.bp[2 + a] = fb(q[2 + a]);
                    break;
            case 2: H.bp[0] = float(q[0]);
                    for (int a = 0; a < 6; ++a) H.bp[1 + a] = fb(q[1 + a]);
                    break;
            case 3: for (int a = 0; a < 3; ++a) {
                        H.bp[a] = float(0.5 / (q[a] * q[a]));
                        H.bp[4 + a] = float(1.0 / (q[a] * q[a]));
                    }
                    H.bp[3] = fb(q[3]);
                    break;
            default: break;
        }
    }
    H.nswarm = c->nswarm;
    H.swarm_off = off();
    if (c->nswarm > 0) {
        for (int k = 0; k < c->nswarm; ++k) {
            for (int a = 0; a < 3; ++a) data.push_back(float(force_to_dev(e * c->swarm_E[3 * k + a])));
            data.push_back(float(c->swarm_Fdt[k]));
        }
    } else {
        for (int a = 0; a < 3; ++a) data.push_back(H.E[a]);
        data.push_back(0.0f);
    }
    while (data.size() % 4) data.push_back(0.0f);
    size_t bytes = sizeof(BlobHdr) + data.size() * 4;
    bytes = (bytes + 15) & ~size_t(15);
    H.bytes = int(bytes);
    c->blob.assign(bytes, 0);
    std::memcpy(c->blob.data(), &H, sizeof(H));
    std::memcpy(c->blob.data() + sizeof(H), data.data(), data.size() * 4);
    if (bytes > c->d_blob_cap) {
        cudaFree(c->d_blob);
        CK(cudaMalloc(&c->d_blob, bytes));
        c->d_blob_cap = bytes;
    }
    CK(cudaMemcpyAsync(c->d_blob, c->blob.data(), bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->blob_dirty = false;
    return PCL_OK;
}

PCL_INTERNAL StepArgs make_args(Ctx* c, double dt, int nsteps, int spill_mode, int sp_in) {
    StepArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        A.xw[s] = S.xw[S.cur];
        A.ps[s] = S.ps[S.cur];
        A.meta[s] = S.meta[S.cur];
        A.in_xw[s] = c->hin_xw[s] ? c->hin_xw[s] : A.xw[s];
        A.in_ps[s] = c->hin_ps[s] ? c->hin_ps[s] : A.ps[s];
        A.in_meta[s] = c->hin_meta[s] ? c->hin_meta[s] : A.meta[s];
        A.hx_xw[s] = c->hx_xw[s];
        A.hx_ps[s] = c->hx_ps[s];
        A.hx_meta[s] = c->hx_meta[s];
        A.hx_cap[s] = c->hx_cap[s];
        A.cap[s] = S.cap;
        A.hist_n[s] = S.hist_n;
        A.hist_w[s] = S.hist_w;
    }
    int sp_out = 1 - sp_in;
    A.sp_in_xw = c->sp_xw[sp_in]; A.sp_in_ps = c->sp_ps[sp_in]; A.sp_in_meta = c->sp_meta[sp_in];
    A.sp_out_xw = c->sp_xw[sp_out]; A.sp_out_ps = c->sp_ps[sp_out]; A.sp_out_meta = c->sp_meta[sp_out];
    A.sp_cap = c->sp_cap;
    A.sp_in_n = c->d_spn + sp_in;
    A.sp_out_n = c->d_spn + sp_out;
    A.ctl = c->d_ctl;
    A.head = &c->d_ctl->head;
    A.blob = c->d_blob;
    for (size_t b = 0; b < c->sb.size(); ++b) A.sb_data[b] = c->sb[b].d_data;
    A.key0 = uint32_t(c->cfg.seed);
    A.key1 = uint32_t(c->cfg.seed >> 32);
    A.dt = dt;
    A.nsteps = nsteps;
    A.spill_mode = spill_mode;
    A.blob_bytes = int(c->blob.size());
    A.wall_xw = c->d_wall_xw; A.wall_pt = c->d_wall_pt; A.wall_meta = c->d_wall_meta;
    A.wall_n = c->d_wall_n; A.wall_cap = c->wall_cap;
    A.general = (c->field_kind != 0 || c->bfield_kind != 0) ? 1 : 0;
    A.learn = c->learn_on ? 1 : 0;
    for (int s = 0; s < 3; ++s) {
        if (c->sp[s].wall_coord >= 0 && c->wall_cap > 0) A.general = 1;
        if (c->sp[s].set && !((c->push_mask >> s) & 1)) A.general = 1;   // a species that is not pushed
    }
    A.event = (c->cfg.classic_step == 0) ? 1 : 0;
    A.stash = c->cfg.stash_entries > 0 ? c->cfg.stash_entries : PCL_STASH_MAX;
    if (c->learn_on) {  // suspended collisions go to queue 0 unless set_lq says otherwise
        A.lq_out_xw = c->lq_xw[0]; A.lq_out_ps = c->lq_ps[0]; A.lq_out_m1 = c->lq_m1[0]; A.lq_out_m2 = c->lq_m2[0];
        A.lq_out_n = c->d_lqn;
        A.lq_cap = c->lq_cap;
    }
    return A;
}

// Suspended-collision queues of a pass: output queue `out`, input queue `in` (-1: none).
PCL_INTERNAL void set_lq(StepArgs& A, Ctx* c, int out, int in) {
    if (!c->learn_on) return;
    A.lq_out_xw = c->lq_xw[out]; A.lq_out_ps = c->lq_ps[out]; A.lq_out_m1 = c->lq_m1[out];
    A.lq_out_m2 = c->lq_m2[out]; A.lq_out_n = c->d_lqn + out;
    if (in >= 0) {
        A.lq_in_xw = c->lq_xw[in]; A.lq_in_ps = c->lq_ps[in]; A.lq_in_m1 = c->lq_m1[in]; A.lq_in_m2 = c->lq_m2[in];
        A.lq_in_n = c->d_lqn + in;
        A.lq_in_y = c->lq_y;
    }
    A.lq_cap = c->lq_cap;
}

PCL_INTERNAL void free_lq(Ctx* c) {
    for (int b = 0; b < 2; ++b) {
        cudaFree(c->lq_xw[b]); cudaFree(c->lq_ps[b]); cudaFree(c->lq_m1[b]); cudaFree(c->lq_m2[b]);
        c->lq_xw[b] = c->lq_ps[b] = nullptr; c->lq_m1[b] = nullptr; c->lq_m2[b] = nullptr;
    }
    cudaFree(c->lq_x); cudaFree(c->lq_yk); cudaFree(c->lq_y); cudaFree(c->d_lqn);
    c->lq_x = c->lq_yk = c->lq_y = nullptr; c->d_lqn = nullptr;
    c->lq_cap = 0; c->lq_nets_cap = 0;
}

// Queues sized for 1/64 of the largest population (at least 64 Ki collisions);
// a full queue makes the step use the table sampler for the excess.
PCL_INTERNAL int ensure_lq(Ctx* c) {
    if (!c->learn_on) return PCL_OK;
    long long capmax = 0;
    for (auto& s : c->sp) capmax = std::max(capmax, s.cap);
    long long want = std::max<long long>(1 << 16, capmax / 64);
    long long nn = std::max<long long>(1, (long long)c->nets.size());
    if (want <= c->lq_cap && nn <= c->lq_nets_cap) return PCL_OK;
    CK(cudaStreamSynchronize(c->stream));
    free_lq(c);
    for (int b = 0; b < 2; ++b) {
        CK(cudaMalloc(&c->lq_xw[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->lq_ps[b], sizeof(float4) * want));
        CK(cudaMalloc(&c->lq_m1[b], sizeof(uint4) * want));
        CK(cudaMalloc(&c->lq_m2[b], sizeof(float4) * want));
    }
    CK(cudaMalloc(&c->lq_x, sizeof(float) * 2 * want));
    CK(cudaMalloc(&c->lq_yk, sizeof(float) * nn * want));
    CK(cudaMalloc(&c->lq_y, sizeof(float) * want));
    CK(cudaMalloc(&c->d_lqn, 2 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
    c->lq_cap = want;
    c->lq_nets_cap = nn;
    return PCL_OK;
}

PCL_INTERNAL int blocks_per_sm(Ctx* c) {
    if (c->cfg.classic_step == 0) return 3;   // the event kernel's stash leaves room for 3 blocks per SM
    int b = c->cfg.blocks_per_sm;
    return (b >= 2 && b <= 4) ? b : 4;
}

PCL_INTERNAL int grid_blocks(Ctx* c) {
    if (c->cfg.grid_blocks > 0) return c->cfg.grid_blocks;
    return blocks_per_sm(c) * c->sm_count;
}

PCL_INTERNAL int block_threads(Ctx* c) {
    int b = c->cfg.block_size > 0 ? c->cfg.block_size : 256;
    return std::min(256, std::max(32, (b / 32) * 32));
}

PCL_INTERNAL int readback(Ctx* c) {
    CK(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PCL_OK;
}

// Device scratch of at least `bytes`, kept across calls (grown by doubling).
PCL_INTERNAL int ensure_scratch(Ctx* c, size_t bytes) {
    if (bytes <= c->scr_bytes) return PCL_OK;
    const size_t nb = std::max(bytes, 2 * c->scr_bytes);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaFree(c->d_scr));
    c->d_scr = nullptr;
    c->scr_bytes = 0;
    CK(cudaMalloc(&c->d_scr, nb));
    c->scr_bytes = nb;
    return PCL_OK;
}

// The per-swarm population cap (pcl_set_swarm_cap) after a launch group:
// count the live particles of each swarm, then roulette the swarms above the
// cap, both on the context stream with the slot count read on the device.
// Removed particles stay as dead slots until the next compaction.
PCL_INTERNAL int apply_swarm_caps(Ctx* c) {
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        if (c->swarm_cap[s] <= 0 || S.cap <= 0) continue;
        const int ns = std::max(1, c->nswarm);
        unsigned int* cnt = c->d_swcnt + 256 * s;
        const int grid = int(std::min<long long>((S.cap + 255) / 256, 4ll * c->sm_count));
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned int) * ns, c->stream));
        k_swarm_count<<<grid, 256, 0, c->stream>>>(S.meta[S.cur], &c->d_ctl->n[s], S.cap, ns, cnt);
        CK(cudaGetLastError());
        k_roulette_cap<<<grid, 256, 0, c->stream>>>(S.xw[S.cur], S.meta[S.cur], &c->d_ctl->n[s], S.cap, cnt, ns,
                                                    (unsigned long long)c->swarm_cap[s], uint32_t(c->cfg.seed),
                                                    uint32_t(c->cfg.seed >> 32));
        CK(cudaGetLastError());
        c->launches += 2;
    }
    return PCL_OK;
}

PCL_INTERNAL CompactArgs make_compact_args(Ctx* c) {
    CompactArgs C;
    std::memset(&C, 0, sizeof(C));
    long long capmax = 0;
    for (int s = 0; s < 3; ++s) {
        SpeciesState& S = c->sp[s];
        int o = 1 - S.cur;
        C.sxw[s] = S.xw[S.cur]; C.sps[s] = S.ps[S.cur]; C.smeta[s] = S.meta[S.cur];
        C.dxw[s] = S.xw[o]; C.dps[s] = S.ps[o]; C.dmeta[s] = S.meta[o];
        C.tile_cnt[s] = c->d_tile_cnt + s * c->tiles_cap;
        C.tile_off[s] = c->d_tile_off + s * c->tiles_cap;
        capmax = std::max(capmax, S.cap);
    }
    C.n = c->d_ctl->n;
    C.n_out = c->d_nnew;
    C.ntiles_max = int(std::max<long long>(1, (capmax + kTile - 1) / kTile));
    return C;
}

// Enqueue the compaction (no host state change: the caller flips buffers).
PCL_INTERNAL cudaError_t enqueue_compact(Ctx* c, const CompactArgs& C) {
    dim3 g(C.ntiles_max, 3);
    k_compact_count<<<g, 256, 0, c->stream>>>(C);
    k_compact_scan<<<3, 1024, 0, c->stream>>>(C);
    k_compact_scatter<<<g, 256, 0, c->stream>>>(C);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(c->d_ctl->n, c->d_nnew, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToDevice,
                           c->stream);
}

PCL_INTERNAL void flip_buffers(Ctx* c) {
    for (int s = 0; s < 3; ++s)
        if (c->sp[s].cap > 0) c->sp[s].cur = 1 - c->sp[s].cur;
    c->steps_since_compact = 0;
}

PCL_INTERNAL int compact_all(Ctx* c) {
    int rc = ensure_tiles(c);
    if (rc) return rc;
    CK(enqueue_compact(c, make_compact_args(c)));
    c->launches += 3;
    flip_buffers(c);
    return PCL_OK;
}

// The learned-sampler round, enqueued with no host read-back (so that it can
// be captured): the networks answer every collision suspended in queue 0 by
// the step and its two spill passes (network inputs, one batched tensor-core
// forward pass per attached network, the pick of each collision's network),
// then a resume pass finishes those collisions and carries the particles to
// the end of the launch, appending its overflow children to spill queue 1
// after what the spill passes left there, and two more spill passes drain
// it.  Every count is read on the device; the resume pass and the passes
// after it use the table sampler for any further collision (no suspension).
PCL_INTERNAL cudaError_t enqueue_learned_round(Ctx* c, double dt, int nsteps, int minb, int threads, size_t smem) {
    const int g = int(std::max<long long>(1, std::min<long long>((c->lq_cap + 255) / 256, 2ll * c->sm_count)));
    const unsigned long long* nq = c->d_lqn;   // queue 0
    k_learn_x<<<g, 256, 0, c->stream>>>(c->lq_ps[0], c->lq_m2[0], nq, c->lq_cap, c->lq_x);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = mlp::infer_multi(c->nets.data(), int(c->nets.size()), c->lq_x, nq, c->lq_cap, c->lq_yk, c->lq_cap,
                             c->stream);
    if (e != cudaSuccess) return e;
    k_learn_pick<<<g, 256, 0, c->stream>>>(c->lq_m2[0], nq, c->lq_cap, c->lq_yk, c->lq_cap, c->pick, c->lq_y);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, nullptr, nullptr);   // work head only
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    StepArgs R = make_args(c, dt, nsteps, 2, 0);   // spill output: queue 1
    set_lq(R, c, 1, 0);
    R.lq_out_n = nullptr;
    // queue-driven passes take any grid: one block per SM, or the persistent
    // grid when the launch has several steps (the resumed particles then carry
    // the rest of the launch's steps)
    const int rgrid = nsteps > 1 ? grid_blocks(c) : c->sm_count;
    if ((e = launch_step(minb, rgrid, threads, smem, c->stream, R)) != cudaSuccess) return e;
    for (int in = 1, pass = 0; pass < 2; ++pass, in = 1 - in) {
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + in, c->d_spn + (1 - in));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        StepArgs P = make_args(c, dt, nsteps, 1, in);
        P.lq_out_n = nullptr;
        if ((e = launch_step(minb, c->sm_count, threads, smem, c->stream, P)) != cudaSuccess) return e;
    }
    c->launches += 8 + ((long long)c->nets.size() + mlp::kMaxNets - 1) / mlp::kMaxNets;
    return cudaSuccess;
}

// Statistics of the learned round of the last launch group (queue 0's count
// read back with the control block).
PCL_INTERNAL void count_learned(Ctx* c) {
    const long long m = std::min<long long>((long long)c->h_lqn[0], c->lq_cap);
    if (m > 0) {
        c->learn_rounds += 1;
        c->learn_suspended += m;
    }
}

// One launch group as a CUDA graph: prologue, step kernel, two spill passes
// (each a no-op when its queue is empty), the compaction when due, and the
// read-back of the control block and spill counts.  Graphs are cached by the
// bytes of every launch parameter, so a replay is identical to a fresh capture.
PCL_INTERNAL int run_group_graph(Ctx* c, const StepArgs& A, const StepArgs& P0, const StepArgs& P1,
                           const CompactArgs* C, int minb, int grid, int threads, size_t smem) {
    std::vector<unsigned char> key;
    auto put = [&key](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + n);
    };
    put(&A, sizeof(A)); put(&P0, sizeof(P0)); put(&P1, sizeof(P1));
    int hdr[4] = {minb, grid, threads, (C ? 1 : 0) | (c->learn_on ? 2 : 0)};
    if (c->learn_on) {   // the learned round's networks and their pick table
        put(c->nets.data(), c->nets.size() * sizeof(void*));
        put(&c->pick, sizeof(c->pick));
        put(&c->lq_cap, sizeof(c->lq_cap));
    }
    put(hdr, sizeof(hdr)); put(&smem, sizeof(smem));
    if (C) put(C, sizeof(*C));
    long long caps[3] = {c->sp[0].cap, c->sp[1].cap, c->sp[2].cap};
    put(caps, sizeof(caps));
    cudaGraphExec_t exec = nullptr;
    for (auto& g : c->graphs)
        if (g.key == key) { exec = g.exec; break; }
    if (!exec) {
        CK(prepare_step(minb, smem, A.general != 0, A.event != 0, A.learn != 0));
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        auto q = [&e](cudaError_t r) { if (e == cudaSuccess) e = r; };
        k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, caps[0], caps[1], caps[2]);
        q(cudaGetLastError());
        q(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
        if (c->learn_on) q(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
        // external records: event-record nodes that fire on every replay, so
        // the step kernel stays timed by events on its own stream
        q(cudaEventRecordWithFlags(c->ev_k0, c->stream, cudaEventRecordExternal));
        q(launch_step(minb, grid, threads, smem, c->stream, A));
        q(cudaEventRecordWithFlags(c->ev_k1, c->stream, cudaEventRecordExternal));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
        q(cudaGetLastError());
        q(launch_step(minb, grid, threads, smem, c->stream, P0));
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
        q(cudaGetLastError());
        q(launch_step(minb, grid, threads, smem, c->stream, P1));
        const long long l0 = c->launches;
        if (c->learn_on) q(enqueue_learned_round(c, A.dt, A.nsteps, minb, threads, smem));
        c->launches = l0;   // counted per replay below
        if (C) q(enqueue_compact(c, *C));
        q(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(Control), cudaMemcpyDeviceToHost, c->stream));
        q(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
        if (c->learn_on)
            q(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              c->stream));
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        CK(e);
        if (c->graphs.size() >= 8) {
            cudaGraphExecDestroy(c->graphs.front().exec);
            c->graphs.erase(c->graphs.begin());
        }
        c->graphs.push_back({std::move(key), exec});
    }
    CK(cudaGraphLaunch(exec, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->graph_launches += 1;
    c->launches += (C ? 11 : 8) +
                   (c->learn_on ? 8 + ((long long)c->nets.size() + mlp::kMaxNets - 1) / mlp::kMaxNets : 0);
    return PCL_OK;
}

// Spill passes: the queue written by the previous pass is the next pass's
// input, starting from spill queue `in`; suspended collisions of these passes
// go to learned queue `lq_out` (-1: none suspended).  *ran = whether any pass ran.
PCL_INTERNAL int drain_spills(Ctx* c, double dt, int nsteps, int threads, size_t smem, int in, int lq_out, bool* ran,
                        const unsigned long long* known_pending) {
    for (int pass = 0; pass < 64; ++pass) {
        unsigned long long pending = 0;
        if (pass == 0 && known_pending) pending = *known_pending;
        else CK(d2h(c, &pending, c->d_spn + in, sizeof(pending)));
        if (pending == 0) return PCL_OK;
        *ran = true;
        k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + in, c->d_spn + (1 - in));
        StepArgs S = make_args(c, dt, nsteps, 1, in);
        if (lq_out >= 0) set_lq(S, c, lq_out, -1);
        else S.lq_out_n = nullptr;   // no suspension in these passes
        CK(launch_step(blocks_per_sm(c), grid_blocks(c), threads, smem, c->stream, S));
        c->launches += 2;
        in = 1 - in;
    }
    return fail(c, PCL_ERR_TIMEOUT, "spill passes did not drain");
}

// One launch of `nsteps` steps of length dt (seconds), plus spill passes and,
// with a learned sampler attached, the learned round.
PCL_INTERNAL int launch_steps(Ctx* c, double dt_si, int nsteps) {
    int rc = build_blob(c);
    if (rc) return rc;
    if ((rc = ensure_spill(c))) return rc;
    if ((rc = ensure_lq(c))) return rc;
    const double dt = t_to_dev(dt_si);
    const int threads = block_threads(c);
    const size_t smem = step_smem_bytes(int(c->blob.size()), threads, c->cfg.classic_step == 0);
    const int period = c->cfg.compaction_period > 0 ? c->cfg.compaction_period : 8;
    const bool graph = c->cfg.use_graph != 0;
    bool compacted = false, host_passes = false;
    StepArgs A = make_args(c, dt, nsteps, 0, 0);
    c->launch_t0.push_back(c->t);   // k_begin advances the device launch counter to match
    unsigned long long pending0 = 0;
    if (graph) {
        const bool due = c->steps_since_compact + nsteps >= period;
        if (due && (rc = ensure_tiles(c))) return rc;
        CompactArgs C;
        if (due) C = make_compact_args(c);
        StepArgs P0 = make_args(c, dt, nsteps, 1, 1), P1 = make_args(c, dt, nsteps, 1, 0);
        if ((rc = run_group_graph(c, A, P0, P1, due ? &C : nullptr, blocks_per_sm(c), grid_blocks(c), threads,
                                  smem)))
            return rc;
        if (due) { flip_buffers(c); compacted = true; }
        pending0 = c->h_spn[1];  // the two in-graph passes leave the last queue written in 1
    } else {
        const int minb = blocks_per_sm(c);
        k_begin<<<1, 64, 0, c->stream>>>(c->d_ctl, c->sp[0].cap, c->sp[1].cap, c->sp[2].cap);
        CK(cudaMemsetAsync(c->d_spn, 0, 2 * sizeof(unsigned long long), c->stream));
        if (c->learn_on) CK(cudaMemsetAsync(c->d_lqn, 0, 2 * sizeof(unsigned long long), c->stream));
        CK(cudaEventRecord(c->ev_k0, c->stream));
        CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, A));
        CK(cudaEventRecord(c->ev_k1, c->stream));
        c->launches += 2;
        if (c->learn_on) {   // the graph's sequence: two spill passes, then the learned round
            StepArgs P0 = make_args(c, dt, nsteps, 1, 1), P1 = make_args(c, dt, nsteps, 1, 0);
            k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 1, c->d_spn + 0);
            CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P0));
            k_begin_spill<<<1, 32, 0, c->stream>>>(c->d_ctl, c->d_spn + 0, c->d_spn + 1);
            CK(launch_step(minb, grid_blocks(c), threads, smem, c->stream, P1));
            c->launches += 4;
            CK(enqueue_learned_round(c, dt, nsteps, minb, threads, smem));
            CK(cudaMemcpyAsync(c->h_lqn, c->d_lqn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c->stream));
        }
        CK(cudaMemcpyAsync(c->h_spn, c->d_spn, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
        if ((rc = readback(c))) return rc;   // the one synchronisation of the group
        pending0 = c->h_spn[1];
    }
    if (c->learn_on) count_learned(c);
    {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1));
        c->k_ms += ms;
        c->k_launches += 1;
        double nstart = 0, nout = 0, ndead = 0;
        for (int s = 0; s < 3; ++s) {
            nstart += double(c->h_ctl->n_start[s]);
            nout += double(c->h_ctl->live_end[nsteps - 1][s]);
            ndead += double(c->h_ctl->dead[s]);
        }
        c->k_bytes += 48.0 * nstart + 48.0 * nout + 4.0 * ndead;
    }
    // leftovers of the in-group passes (rare): host-driven passes, table sampler only
    if ((rc = drain_spills(c, dt, nsteps, threads, smem, 1, -1, &host_passes, &pending0))) return rc;
    // the last read-back holds the final counters unless host passes ran after it
    if (host_passes && (rc = readback(c))) return rc;
    if (c->h_ctl->timeout) return fail(c, PCL_ERR_TIMEOUT, "table staging wait timed out");
    c->t += dt_si * nsteps;
    c->steps += nsteps;
    for (int k = 0; k < nsteps; ++k) c->particle_steps += (long long)c->h_ctl->live_start[k];
    for (int s = 0; s < 3; ++s) c->live[s] = (long long)c->h_ctl->live_end[nsteps - 1][s];
    if (!compacted) {
        c->steps_since_compact += nsteps;
        if (c->steps_since_compact >= period) {
            if ((rc = compact_all(c))) return rc;
        }
    }
    if (c->h_ctl->err[PCL_E_CAPACITY] > 0) return fail(c, PCL_ERR_CAPACITY, "population capacity exceeded");
    return PCL_OK;
}

PCL_INTERNAL int check_species(Ctx* c, int s) {
    if (s < 0 || s >= 3) return fail(c, PCL_ERR_INVALID, "species out of range");
    return PCL_OK;
}


PCL_INTERNAL int get_n(Ctx* c, int species, long long& n) {
    unsigned long long nn = 0;
    CK(d2h(c, &nn, &c->d_ctl->n[species], sizeof(nn)));
    n = std::min<long long>((long long)nn, c->sp[species].cap);
    return PCL_OK;
}

}  // namespace pcl

using namespace pcl;

// =============================================================== C ABI ===
extern "C" {


const char* pcl_version(void) { return "particulator_gb300 0.1 (sm_103a)"; }

int pcl_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

const char* pcl_last_error(void* ctx) {
    if (!ctx) return noalloc_last_error();
    return static_cast<Ctx*>(ctx)->last_error.c_str();
}

int pcl_create(const pcl_config* cfg, void** out) {
    if (!cfg || !out) return PCL_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PCL_ERR_CUDA;
    if (cfg->device < 0 || cfg->device >= ndev) return PCL_ERR_INVALID;
    if (cfg->steps_per_launch > PCL_MAX_STEPS_PER_LAUNCH) return PCL_ERR_INVALID;
    if (cfg->stash_entries < 0 || cfg->stash_entries > PCL_STASH_MAX) return PCL_ERR_INVALID;
    Ctx* c = new Ctx();
    c->cfg = *cfg;
    c->device = cfg->device;
    if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return PCL_ERR_CUDA; }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_ctl, sizeof(Control)) != cudaSuccess ||
        cudaMallocHost(&c->h_ctl, sizeof(Control)) != cudaSuccess ||
        cudaMallocHost(&c->h_spn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&c->h_lqn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_spn, 2 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_nnew, 3 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&c->d_mom, 16 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->d_swcnt, 3 * 256 * sizeof(unsigned int)) != cudaSuccess ||
        cudaEventCreate(&c->ev_k0) != cudaSuccess || cudaEventCreate(&c->ev_k1) != cudaSuccess ||
        cudaEventCreate(&c->ev_t0) != cudaSuccess || cudaEventCreate(&c->ev_t1) != cudaSuccess) {
        pcl_destroy(c);
        return PCL_ERR_CUDA;
    }
    cudaMemset(c->d_ctl, 0, sizeof(Control));
    cudaMemset(c->d_spn, 0, 2 * sizeof(unsigned long long));
    std::memset(c->h_ctl, 0, sizeof(Control));
    cudaDeviceSynchronize();
    *out = c;
    return PCL_OK;
}

void pcl_destroy(void* ctx) {
    if (!ctx) return;
    Ctx* c = static_cast<Ctx*>(ctx);
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& s : c->sp) free_species_buffers(s);
    for (auto& t : c->sb) cudaFree(t.d_data);
    for (int b = 0; b < 2; ++b) { cudaFree(c->sp_xw[b]); cudaFree(c->sp_ps[b]); cudaFree(c->sp_meta[b]); }
    cudaFree(c->d_spn); cudaFree(c->d_blob); cudaFree(c->d_ctl); cudaFree(c->d_tile_cnt);
    cudaFree(c->d_tile_off); cudaFree(c->d_nnew); cudaFree(c->d_mom); cudaFree(c->d_scr); cudaFree(c->d_swcnt);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    if (c->h_spn) cudaFreeHost(c->h_spn);
    if (c->h_lqn) cudaFreeHost(c->h_lqn);
    for (cudaEvent_t e : c->io_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : c->io_tev) cudaEventDestroy(e);
    if (c->io_join) cudaEventDestroy(c->io_join);
    if (c->s_h2d) cudaStreamDestroy(c->s_h2d);
    if (c->s_d2h) cudaStreamDestroy(c->s_d2h);
    if (c->s_cmp) cudaStreamDestroy(c->s_cmp);
    cudaFree(c->d_heads);
    free_lq(c);
    cudaFree(c->d_wall_xw); cudaFree(c->d_wall_pt); cudaFree(c->d_wall_meta); cudaFree(c->d_wall_n);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    for (cudaEvent_t ev : {c->ev_k0, c->ev_k1, c->ev_t0, c->ev_t1})
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int pcl_set_species(void* ctx, int species, double energy_cut, int64_t capacity, int flags) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (capacity < 0 || capacity >= (1ll << 31)) return fail(c, PCL_ERR_INVALID, "capacity out of range");
    if (!(energy_cut >= 0)) return fail(c, PCL_ERR_INVALID, "energy cut must be >= 0");
    CK(cudaSetDevice(c->device));
    SpeciesState& S = c->sp[species];
    CK(cudaStreamSynchronize(c->stream));
    free_species_buffers(S);
    S.set = true;
    S.cut = energy_cut;
    S.flags = flags;
    S.cap = (flags & PCL_SPECIES_TALLY_ONLY) ? 0 : capacity;
    S.cur = 0;
    if (S.cap > 0) {
        for (int b = 0; b < 2; ++b) {
            CK(cudaMalloc(&S.xw[b], sizeof(float4) * S.cap));
            CK(cudaMalloc(&S.ps[b], sizeof(float4) * S.cap));
            CK(cudaMalloc(&S.meta[b], sizeof(uint4) * S.cap));
        }
    }
    unsigned long long zero = 0;
    CK(h2d(c, &c->d_ctl->n[species], &zero, sizeof(zero)));
    c->live[species] = 0;
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_collision_table(void* ctx, int species, int order, int nproc, int nintervals, double xmax,
                            const double* rate, const double* ratebound, const pcl_process* procs) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (order < 1 || order > PCL_MAX_ORDER || nproc < 0 || nproc > PCL_MAX_PROC || nintervals < 1 ||
        nintervals > PCL_MAX_INTERVALS || !(xmax > 0) || !ratebound || (nproc > 0 && (!rate || !procs)))
        return fail(c, PCL_ERR_INVALID, "bad collision table");
    SpeciesState& S = c->sp[species];
    const int nI = nintervals + 1;
    S.table_kind = 0;
    S.order = order; S.nproc = nproc; S.nint = nintervals; S.xmax = xmax;
    S.rate.assign(rate, rate + size_t(order) * nproc * nI);
    if (nproc == 0) S.rate.clear();
    S.rb.assign(ratebound, ratebound + size_t(order) * nI);
    S.procs.assign(procs, procs + nproc);
    S.sb_index.assign(nproc, -1);
    CK(cudaSetDevice(c->device));
    for (int j = 0; j < nproc; ++j) {
        const pcl_process& P = procs[j];
        if (P.kind < PCL_PROC_MOLLER || P.kind > PCL_PROC_ATTACHMENT)
            return fail(c, PCL_ERR_UNSUPPORTED, "unsupported process kind");
        if (P.kind == PCL_PROC_SELTZER_BERGER) {
            if (!P.aux0 || !P.aux2 || P.naux < 2 || P.naux2 < 2)
                return fail(c, PCL_ERR_INVALID, "Seltzer-Berger process needs log_energy and data");
            int found = -1;
            // one device table per distinct inverse-CDF content (the reference's
            // SeltzerBerger struct carries no Z, and every Z shares one energy grid)
            for (size_t b = 0; b < c->sb.size(); ++b)
                if (c->sb[b].ne == P.naux && c->sb[b].ncum == P.naux2 &&
                    c->sb[b].log_energy == std::vector<double>(P.aux0, P.aux0 + P.naux) &&
                    c->sb[b].data == std::vector<double>(P.aux2, P.aux2 + size_t(P.naux) * P.naux2))
                    found = int(b);
            if (found < 0) {
                if (c->sb.size() >= PCL_MAX_SB) return fail(c, PCL_ERR_UNSUPPORTED, "too many SB tables");
                SBTable T;
                T.Z = P.Z; T.ne = P.naux; T.ncum = P.naux2;
                T.log_energy.assign(P.aux0, P.aux0 + P.naux);
                T.data.assign(P.aux2, P.aux2 + size_t(P.naux) * P.naux2);
                std::vector<float> f(size_t(T.ne) * T.ncum);
                for (size_t q = 0; q < f.size(); ++q) f[q] = float(P.aux2[q]);
                CK(cudaMalloc(&T.d_data, f.size() * sizeof(float)));
                CK(h2d(c, T.d_data, f.data(), f.size() * sizeof(float)));
                c->sb.push_back(T);
                found = int(c->sb.size()) - 1;
            }
            S.sb_index[j] = found;
        }
        if (P.kind == PCL_PROC_PHOTOELECTRIC && P.nparam < 1)
            return fail(c, PCL_ERR_INVALID, "photoelectric process needs binding energies");
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_linear_table(void* ctx, int species, int nproc, int n, double e0, double e1, const double* rate,
                         const double* ratebound, int nrb, const pcl_process* procs) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nproc < 0 || nproc > PCL_MAX_PROC || n < 2 || !(e1 > e0) || !ratebound || (nrb != 1 && nrb != n) ||
        (nproc > 0 && (!rate || !procs)))
        return fail(c, PCL_ERR_INVALID, "bad linear collision table");
    for (int j = 0; j < nproc; ++j)
        if (procs[j].kind != PCL_PROC_ELASTIC && procs[j].kind != PCL_PROC_EXCITATION &&
            procs[j].kind != PCL_PROC_NULL_COLLISION && procs[j].kind != PCL_PROC_REL_COULOMB &&
            procs[j].kind != PCL_PROC_IONIZATION && procs[j].kind != PCL_PROC_ATTACHMENT)
            return fail(c, PCL_ERR_UNSUPPORTED, "process kind not supported on a linear-grid table");
    SpeciesState& S = c->sp[species];
    S.table_kind = 1;
    S.nproc = nproc; S.order = 1; S.nint = 1; S.xmax = e1;
    S.lin_n = n; S.lin_e0 = e0; S.lin_e1 = e1;
    S.rate.assign(rate, rate + size_t(nproc) * n);
    S.rb.resize(n);
    for (int i = 0; i < n; ++i) S.rb[i] = ratebound[nrb == 1 ? 0 : i];
    S.procs.assign(procs, procs + nproc);
    S.sb_index.assign(nproc, -1);
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_forcing(void* ctx, const double E[3], const double B[3], int cl_order, int cl_k, double cl_xmax,
                    const double* cl_ec, const double* cl_pc) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !E || !B) return PCL_ERR_INVALID;
    if (cl_order < 0 || cl_order > PCL_MAX_ORDER) return fail(c, PCL_ERR_INVALID, "bad continuum order");
    for (int a = 0; a < 3; ++a) { c->E[a] = E[a]; c->B[a] = B[a]; }
    c->cl_order = cl_order;
    if (cl_order > 0) {
        if (cl_k < 1 || cl_k > PCL_MAX_INTERVALS || !(cl_xmax > 0) || !cl_ec || !cl_pc)
            return fail(c, PCL_ERR_INVALID, "bad continuum-loss table");
        c->cl_k = cl_k;
        c->cl_xmax = cl_xmax;
        c->cl_ec.assign(cl_ec, cl_ec + size_t(cl_order) * (cl_k + 1));
        c->cl_pc.assign(cl_pc, cl_pc + size_t(cl_order) * (cl_k + 1));
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_field(void* ctx, int kind, const double* params, int nparams) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    static const int need[4] = {0, 5, 7, 4};
    if (kind < 0 || kind > 3 || nparams < need[kind] || (need[kind] > 0 && !params))
        return fail(c, PCL_ERR_INVALID, "field kind or parameters");
    if (kind == 3 && !(params[0] > 0 && params[1] > 0 && params[2] > 0))
        return fail(c, PCL_ERR_INVALID, "confined double layer widths must be > 0");
    c->field_kind = kind;
    for (int i = 0; i < 8; ++i) c->field_p[i] = (i < need[kind]) ? params[i] : 0.0;
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_bfield(void* ctx, int kind, const double* params, int nparams) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    static const int need[4] = {0, 5, 7, 4};
    if (kind < 0 || kind > 3 || nparams < need[kind] || (need[kind] > 0 && !params))
        return fail(c, PCL_ERR_INVALID, "field kind or parameters");
    if (kind == 3 && !(params[0] > 0 && params[1] > 0 && params[2] > 0))
        return fail(c, PCL_ERR_INVALID, "confined double layer widths must be > 0");
    c->bfield_kind = kind;
    for (int i = 0; i < 8; ++i) c->bfield_p[i] = (i < need[kind]) ? params[i] : 0.0;
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_set_push_mask(void* ctx, int pushed, int field, int loss) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (pushed < 0 || pushed > 7 || field < 0 || field > 7 || loss < 0 || loss > 7)
        return fail(c, PCL_ERR_INVALID, "species masks are 3-bit");
    c->push_mask = pushed;
    c->field_mask = field;
    c->loss_mask = loss;
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_advance(void* ctx, double tfinal) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (!(tfinal > c->t)) return fail(c, PCL_ERR_INVALID, "tfinal must exceed the current time");
    bool any = false;
    for (auto& s : c->sp) any = any || s.set;
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    return launch_steps(c, tfinal - c->t, 1);
}

int pcl_run(void* ctx, double tfinal, double dt, const pcl_run_opts* opts, pcl_tallies* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (!(dt > 0)) return fail(c, PCL_ERR_INVALID, "dt must be > 0");
    CK(cudaSetDevice(c->device));
    const int K = std::max(1, c->cfg.steps_per_launch);
    // run.jl:6-27 steps while t < tfinal; the step count is fixed once, with a
    // tolerance, so that accumulated rounding of the clock never adds a step
    const long long total = (long long)std::ceil((tfinal - c->t) / dt - 1e-6);
    long long done = 0;
    const bool target = opts && opts->target_species >= 0 && opts->target_species < 3;
    double g_ext = 0.0;   // largest (ismax) or smallest per-step live ratio of the target species so far
    while (done < total) {
        // advance!, droplow!, onstep (population target)
        int ns = int(std::min<long long>(K, total - done));
        if (opts && opts->max_steps > 0) ns = int(std::min<long long>(ns, opts->max_steps - done));
        if (ns <= 0) break;
        if (target && ns > 1) {
            // run.jl:6-27 tests the target after every step.  A launch of ns
            // steps can only stop at its end, so near the target the launches
            // shrink: ns is the number of steps that the fastest per-step change
            // seen so far, with a margin, needs to reach the target (one step
            // until a change has been seen).
            const double live = double(c->live[opts->target_species]), n = double(opts->target_n);
            int m = 1;
            if (g_ext > 0.0) {
                if (opts->target_ismax) {
                    const double g = std::max(g_ext, 1.0) * 1.01;
                    m = (g_ext <= 1.0) ? ns : int(std::floor(std::log(n / (1.05 * live + 1.0)) / std::log(g)));
                } else {
                    const double g = std::min(g_ext, 1.0) * 0.99;
                    m = (g_ext >= 1.0) ? ns
                                       : int(std::floor(std::log((0.95 * live) / std::max(n, 0.5)) / -std::log(g)));
                }
            }
            ns = std::max(1, std::min(ns, m));
        }
        const long long live0 = target ? c->live[opts->target_species] : 0;
        int rc = launch_steps(c, dt, ns);
        if (rc || (rc = apply_swarm_caps(c))) return rc;
        if (target) {
            double prev = double(std::max<long long>(live0, 1));
            for (int k = 0; k < ns; ++k) {
                const double cur = double(c->h_ctl->live_end[k][opts->target_species]);
                const double r = std::max(cur, 1.0) / prev;
                g_ext = (g_ext == 0.0) ? r : (opts->target_ismax ? std::max(g_ext, r) : std::min(g_ext, r));
                prev = std::max(cur, 1.0);
            }
        }
        done += ns;
        if (done == total && std::fabs(c->t - tfinal) < 1e-6 * dt) c->t = tfinal;
        if (opts && opts->target_species >= 0 && opts->target_species < 3) {
            long long live = c->live[opts->target_species];
            bool cont = opts->target_ismax ? (live < opts->target_n) : (live > opts->target_n);
            if (!cont) break;
        }
        if (opts && opts->max_steps > 0 && done >= opts->max_steps) break;
    }
    if (out) return pcl_get_tallies(ctx, out);
    return PCL_OK;
}

int pcl_get_tallies(void* ctx, pcl_tallies* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    int rc = readback(c);
    if (rc) return rc;
    std::memset(out, 0, sizeof(*out));
    const Control& C = *c->h_ctl;
    out->t = c->t;
    out->steps = c->steps;
    out->particle_steps = c->particle_steps;
    for (int s = 0; s < 3; ++s) {
        out->n[s] = std::min<long long>((long long)C.n[s], c->sp[s].cap);
        out->live[s] = c->live[s];
        for (int j = 0; j < PCL_MAX_PROC; ++j) out->collisions[s][j] = (long long)C.coll[s][j];
        out->nulls[s] = (long long)C.nulls[s];
        out->spawned[s] = (long long)C.spawned[s];
        out->tally_count[s] = (long long)C.tally_count[s];
        out->tally_w[s] = C.tally_w[s];
        out->tally_wE[s] = e_to_si(C.tally_wE[s]);
    }
    for (int e = 0; e < PCL_NERR; ++e) out->errors[e] = (long long)C.err[e];
    return PCL_OK;
}

int pcl_reset_tallies(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    int rc = readback(c);
    if (rc) return rc;
    Control keep = *c->h_ctl;
    Control z;
    std::memset(&z, 0, sizeof(z));
    for (int s = 0; s < 3; ++s) z.n[s] = keep.n[s];
    CK(h2d(c, c->d_ctl, &z, sizeof(z)));
    c->particle_steps = 0;
    for (auto& S : c->sp) {
        if (S.hist_bins > 0) {
            CK(cudaMemsetAsync(S.hist_n, 0, sizeof(unsigned long long) * S.hist_bins, c->stream));
            CK(cudaMemsetAsync(S.hist_w, 0, sizeof(double) * S.hist_bins, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
    }
    return PCL_OK;
}

int pcl_moments(void* ctx, int species, double out[10]) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !out) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    long long slots = 0;
    if (S.cap > 0 && (rc = get_n(c, species, slots))) return rc;
    CK(cudaMemsetAsync(c->d_mom, 0, 10 * sizeof(double), c->stream));
    if (slots > 0) {
        int blocks = int(std::min<long long>(4 * c->sm_count, (slots + 255) / 256));
        k_moments<<<blocks, 256, 0, c->stream>>>(S.xw[S.cur], S.ps[S.cur], S.meta[S.cur], slots, species,
                                                   c->d_mom);
        CK(cudaGetLastError());
    }
    double h[10];
    CK(cudaMemcpyAsync(h, c->d_mom, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 8; ++q) out[q] = h[q];
    out[1] = e_to_si(h[1]);
    out[8] = e_to_si(h[8]);
    unsigned long long live;
    std::memcpy(&live, &h[9], 8);
    out[9] = double(live);
    return PCL_OK;
}

int pcl_compact(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    int rc = compact_all(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    return PCL_OK;
}

int pcl_set_tally_histogram(void* ctx, int species, int nbins, double emin, double emax) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    if (nbins < 0 || nbins > (1 << 16) || (nbins > 0 && !(emin > 0 && emax > emin)))
        return fail(c, PCL_ERR_INVALID, "bad histogram");
    SpeciesState& S = c->sp[species];
    CK(cudaSetDevice(c->device));
    cudaFree(S.hist_n); cudaFree(S.hist_w);
    S.hist_n = nullptr; S.hist_w = nullptr;
    S.hist_bins = nbins; S.hist_emin = emin; S.hist_emax = emax;
    if (nbins > 0) {
        CK(cudaMalloc(&S.hist_n, sizeof(unsigned long long) * nbins));
        CK(cudaMalloc(&S.hist_w, sizeof(double) * nbins));
        CK(cudaMemsetAsync(S.hist_n, 0, sizeof(unsigned long long) * nbins, c->stream));
        CK(cudaMemsetAsync(S.hist_w, 0, sizeof(double) * nbins, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->blob_dirty = true;
    return PCL_OK;
}

int pcl_get_tally_histogram(void* ctx, int species, int nbins, int64_t* counts, double* weights) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    int rc = check_species(c, species);
    if (rc) return rc;
    SpeciesState& S = c->sp[species];
    if (nbins != S.hist_bins) return fail(c, PCL_ERR_INVALID, "bin count mismatch");
    if (nbins == 0) return PCL_OK;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (counts) CK(d2h(c, counts, S.hist_n, sizeof(int64_t) * nbins));
    if (weights) CK(d2h(c, weights, S.hist_w, sizeof(double) * nbins));
    return PCL_OK;
}

int pcl_sync(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaGetLastError());
    return PCL_OK;
}

int pcl_test_timeout(void* ctx, int max_iters) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || max_iters < 1 || max_iters > (1 << 20)) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    k_test_wait<<<1, 64, 0, c->stream>>>(c->d_ctl, max_iters);
    CK(cudaGetLastError());
    int rc = readback(c);
    if (rc) return rc;
    if (c->h_ctl->timeout) {   // the context stays usable: clear the flag, report the status
        CK(cudaMemsetAsync(&c->d_ctl->timeout, 0, sizeof(c->d_ctl->timeout), c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return fail(c, PCL_ERR_TIMEOUT, "bounded wait gave up (test hook)");
    }
    return PCL_OK;
}

int pcl_timer_start(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaEventRecord(c->ev_t0, c->stream));
    return PCL_OK;
}

int pcl_timer_stop(void* ctx, double* ms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !ms) return PCL_ERR_INVALID;
    CK(cudaSetDevice(c->device));
    CK(cudaEventRecord(c->ev_t1, c->stream));
    CK(cudaEventSynchronize(c->ev_t1));
    float f = 0.0f;
    CK(cudaEventElapsedTime(&f, c->ev_t0, c->ev_t1));
    *ms = f;
    return PCL_OK;
}

int pcl_kernel_stats(void* ctx, double* step_kernel_ms, int64_t* step_launches, int64_t* launches,
                     double* step_bytes, int reset) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return PCL_ERR_INVALID;
    if (step_kernel_ms) *step_kernel_ms = c->k_ms;
    if (step_launches) *step_launches = c->k_launches;
    if (launches) *launches = c->launches;
    if (step_bytes) *step_bytes = c->k_bytes;
    if (reset) { c->k_ms = 0; c->k_launches = 0; c->launches = 0; c->k_bytes = 0; }
    return PCL_OK;
}

int pcl_autotune(void* ctx, double dt, int32_t steps_budget, pcl_tune_result* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !(dt > 0) || steps_budget < 16) return PCL_ERR_INVALID;
    bool any = false;
    for (auto& sp : c->sp) any = any || sp.set;
    if (!any) return fail(c, PCL_ERR_STATE, "no species set");
    CK(cudaSetDevice(c->device));
    // step kernel: 0 = event, 2-4 = classic with that many blocks per SM
    const int bps_c[] = {0, 2, 3, 4}, k_c[] = {1, 2, 4, 8, 16, 32, 64}, per_c[] = {2, 4, 8, 16, 32}, g_c[] = {0, 1};
    const int ntrials = 4 + 7 + 5 + 2 + 3;
    // steps per trial: a multiple of the largest steps-per-launch tried (64),
    // so that every trial is a whole number of launches; a budget below
    // ntrials x 64 steps ends the search early (the candidates are tried in
    // the order above, then the other step kernels once more at the chosen
    // steps per launch, compaction period and graph setting)
    int len = std::max(64, (steps_budget / ntrials) / 64 * 64);
    pcl_config best = c->cfg;
    best.blocks_per_sm = (c->cfg.classic_step == 0) ? 4 : blocks_per_sm(c);
    if (best.steps_per_launch < 1) best.steps_per_launch = 1;
    if (best.compaction_period < 1) best.compaction_period = 8;
    double best_rate = -1.0;
    int trials = 0, done = 0;
    auto trial = [&](const pcl_config& cfg, double& rate) -> int {
        c->cfg = cfg;
        int rc = compact_all(c);   // every trial starts from a compacted population
        if (rc) return rc;
        const long long ps0 = c->particle_steps;
        CK(cudaEventRecord(c->ev_t0, c->stream));
        int left = len;
        while (left > 0) {
            int ns = std::min(left, std::max(1, cfg.steps_per_launch));
            if ((rc = launch_steps(c, dt, ns))) return rc;
            left -= ns;
        }
        CK(cudaEventRecord(c->ev_t1, c->stream));
        CK(cudaEventSynchronize(c->ev_t1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1));
        rate = double(c->particle_steps - ps0) / (double(ms) * 1e-3);
        done += len;
        ++trials;
        return PCL_OK;
    };
    auto consider = [&](pcl_config cfg) -> int {
        if (done + len > steps_budget) return PCL_OK;
        double r = 0.0;
        int rc = trial(cfg, r);
        if (rc) return rc;
        if (r > best_rate) { best_rate = r; best = cfg; }
        return PCL_OK;
    };
    int rc = PCL_OK;
    for (int v : bps_c) {
        pcl_config q = best;
        q.classic_step = (v == 0) ? 0 : 1;
        q.blocks_per_sm = (v == 0) ? 4 : v;
        if ((rc = consider(q))) return rc;
    }
    const pcl_config after_bps = best;
    for (int v : k_c) { pcl_config q = after_bps; q.steps_per_launch = v; if ((rc = consider(q))) return rc; }
    const pcl_config after_k = best;
    for (int v : per_c) { pcl_config q = after_k; q.compaction_period = v; if ((rc = consider(q))) return rc; }
    const pcl_config after_p = best;
    for (int v : g_c) { pcl_config q = after_p; q.use_graph = v; if ((rc = consider(q))) return rc; }
    // the best kernel depends on the launch shape: a second pass over the others
    const pcl_config after_g = best;
    for (int v : bps_c) {
        const bool same = (v == 0) ? after_g.classic_step == 0 : (after_g.classic_step != 0 && after_g.blocks_per_sm == v);
        if (same) continue;
        pcl_config q = after_g;
        q.classic_step = (v == 0) ? 0 : 1;
        q.blocks_per_sm = (v == 0) ? 4 : v;
        if ((rc = consider(q))) return rc;
    }
    c->cfg = best;
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->blocks_per_sm = best.classic_step ? best.blocks_per_sm : 0;
        out->steps_per_launch = best.steps_per_launch;
        out->compaction_period = best.compaction_period;
        out->use_graph = best.use_graph;
        out->rate = best_rate;
        out->trials = trials;
        out->steps = done;
    }
    return PCL_OK;
}

int pcl_set_launch(void* ctx, int32_t bps, int32_t spl, int32_t period, int32_t use_graph) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !(bps == 0 || (bps >= 2 && bps <= 4)) || spl < 1 || spl > PCL_MAX_STEPS_PER_LAUNCH || period < 1 ||
        (use_graph != 0 && use_graph != 1))
        return PCL_ERR_INVALID;
    c->cfg.classic_step = (bps == 0) ? 0 : 1;
    c->cfg.blocks_per_sm = (bps == 0) ? 4 : bps;
    c->cfg.steps_per_launch = spl;
    c->cfg.compaction_period = period;
    c->cfg.use_graph = use_graph;
    return PCL_OK;
}

}  // extern "C"
