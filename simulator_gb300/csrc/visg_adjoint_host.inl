// Adjoint of the fused step: forward with checkpoints, backward with recomputation.
// Included by visg_api.cu (member functions of Engine).
//
// visg_forward starts from the simulator's current state, runs the differentiable
// trajectory in FP64 (launch_step_f64: the same algorithm as the float step, in
// double) and keeps its state (x, x_old, contact normal) every `ckpt` steps; at the
// end the simulator's float state is set to the FP64 final state rounded to float.
// visg_backward walks the segments from the last to the first: it restores the
// segment's checkpoint, replays its steps (deterministic, so the contact set is the
// forward pass's), recording every intermediate state, then runs the two adjoint
// kernels per step in reverse.

int Engine::forward(int nsteps, int ckpt) {
    if (!finalized) return fail(VISG_ERR_STATE, "not finalized");
    if (G != 1) return fail(VISG_ERR_UNSUPPORTED, "the adjoint runs on a single-garment simulator");
    if (nsteps < 1 || ckpt < 1) return fail(VISG_ERR_INVALID_ARG, "nsteps and checkpoint_every must be >= 1");
    if (!adj.rev) {
        // reverse entry of every directed spring (same list, k-th duplicate to k-th)
        std::vector<uint32_t> hrev(E > 0 ? E : 1, 0xffffffffu);
        std::vector<uint2> ent(E > 0 ? E : 1);
        CU(cudaMemcpy(ent.data(), d_ent, E * sizeof(uint2), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < N; ++i) {
            const uint32_t rp = h_rowp[i] & ROW_MASK, re = h_rowp[i + 1] & ROW_MASK;
            for (uint32_t e = rp; e < re; ++e) {
                if (hrev[e] != 0xffffffffu) continue;
                const uint32_t j = ent[e].x & END_MASK, l = ent[e].x >> LIST_SHIFT;
                const uint32_t jp = h_rowp[j] & ROW_MASK, je = h_rowp[j + 1] & ROW_MASK;
                bool found = false;
                for (uint32_t f = jp; f < je && !found; ++f)
                    if (f != e && (ent[f].x & END_MASK) == (uint32_t)i && (ent[f].x >> LIST_SHIFT) == l &&
                        hrev[f] == 0xffffffffu) {
                        hrev[e] = f;
                        hrev[f] = e;
                        found = true;
                    }
                if (!found)
                    return fail(VISG_ERR_UNSUPPORTED,
                                "the adjoint needs a symmetric spring graph (i->j and j->i in the same list)");
            }
        }
        CU(cudaMalloc((void**)&adj.rev, (size_t)std::max<int64_t>(E, 1) * 4));
        CU(cudaMemcpy(adj.rev, hrev.data(), (size_t)std::max<int64_t>(E, 1) * 4, cudaMemcpyHostToDevice));
    }
    for (auto* q : adj.ck) cudaFree(q);
    adj.ck.clear();
    if (adj.rec) {
        cudaFree(adj.rec);
        adj.rec = nullptr;
    }
    const size_t n3 = 3 * (size_t)N, st = 9 * (size_t)N;
    const int nck = (nsteps + ckpt - 1) / ckpt;
    for (int c = 0; c < nck; ++c) {
        double* q = nullptr;
        CU(cudaMalloc((void**)&q, st * sizeof(double)));
        adj.ck.push_back(q);
    }
    if (!adj.s64) CU(cudaMalloc((void**)&adj.s64, 15 * (size_t)N * sizeof(double)));
    CU(cudaMalloc((void**)&adj.rec, (size_t)(ckpt + 1) * st * sizeof(double)));
    if (!adj.lam) CU(cudaMalloc((void**)&adj.lam, 12 * (size_t)N * sizeof(double)));
    if (!adj.G) CU(cudaMalloc((void**)&adj.G, n3 * sizeof(double)));
    if (!adj.dk) CU(cudaMalloc((void**)&adj.dk, (size_t)std::max<int64_t>(E, 1) * sizeof(double)));
    if (!adj.dsc) CU(cudaMalloc((void**)&adj.dsc, 3 * sizeof(double)));
    if (adj.contacts) cudaFree(adj.contacts);
    adj.contacts = nullptr;
    CU(cudaMalloc((void**)&adj.contacts, (size_t)nsteps * sizeof(unsigned)));
    CU(cudaMemsetAsync(adj.contacts, 0, (size_t)nsteps * sizeof(unsigned), stream));
    adj.ckpt = ckpt;
    adj.nsteps = nsteps;
    adj.ready = false;
    // FP64 state: s64 = [x0 | xo0 | x1 | xo1 | n], widened from the float state
    CU(launch_unpack_state(d_state[cur], d_state[cur ^ 1], d_normal, N, d_stage, d_stage + n3, d_stage + 2 * n3,
                           stream));
    CU(launch_widen(d_stage, adj.s64, 2 * (int64_t)n3, stream));
    CU(launch_widen(d_stage + 2 * n3, adj.s64 + 4 * n3, (int64_t)n3, stream));
    int c = 0;
    for (int s = 0; s < nsteps; ++s) {
        if (s % ckpt == 0) CU(save64(c, adj.ck[s / ckpt]));
        CU(step64(c, adj.contacts + s));
        c ^= 1;
    }
    // the simulator continues from the FP64 final state, rounded to float
    CU(launch_narrow(adj.s64 + 2 * (size_t)c * n3, d_stage, 2 * (int64_t)n3, stream));
    CU(launch_narrow(adj.s64 + 4 * n3, d_stage + 2 * n3, (int64_t)n3, stream));
    CU(launch_pack_state(d_state[cur], d_state[cur ^ 1], d_normal, N, d_stage, d_stage + n3, d_stage + 2 * n3, p.dt,
                         step_params().drec, step_params().dmax, d_wild, stream));
    if (int r = sync()) return r;
    adj.ready = true;
    return VISG_OK;
}

// one FP64 step from buffer c of s64 into buffer c ^ 1 (normals in place); with
// `contacts`, the step's projected vertices are counted there
cudaError_t Engine::step64(int c, unsigned* contacts) {
    const size_t n3 = 3 * (size_t)N;
    const double* x = adj.s64 + 2 * (size_t)c * n3;
    double* y = adj.s64 + 2 * (size_t)(c ^ 1) * n3;
    const bool coll = p.collide && any_body;
    return launch_step_f64(x, x + n3, y, y + n3, adj.s64 + 4 * n3, d_rowp, d_ent, d_k, d_views,
                           coll ? bvh[0].verts : nullptr, coll ? bvh[0].tris : nullptr, step_params(),
                           (variant() & SV_REFV) ? 1 : 0, coll ? 1 : 0, (int)N, d_err, contacts, stream);
}

// vertices projected in each step of the last forward pass
int Engine::forward_contacts(int64_t* counts, int n) {
    if (!adj.ready) return fail(VISG_ERR_STATE, "visg_forward_contacts needs a visg_forward first");
    if (!counts || n < 0 || n > adj.nsteps) return fail(VISG_ERR_INVALID_ARG, "counts NULL or n out of range");
    std::vector<unsigned> h((size_t)std::max(n, 1));
    if (n > 0) CU(cudaMemcpyAsync(h.data(), adj.contacts, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    if (int r = sync()) return r;
    for (int k = 0; k < n; ++k) counts[k] = (int64_t)h[k];
    return VISG_OK;
}

// [x | xo | n] of FP64 buffer c into dst (9N doubles)
cudaError_t Engine::save64(int c, double* dst) {
    const size_t n3 = 3 * (size_t)N;
    cudaError_t e = cudaMemcpyAsync(dst, adj.s64 + 2 * (size_t)c * n3, 2 * n3 * sizeof(double),
                                    cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(dst + 2 * n3, adj.s64 + 4 * n3, n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream);
}

cudaError_t Engine::load64(const double* src) {
    const size_t n3 = 3 * (size_t)N;
    cudaError_t e = cudaMemcpyAsync(adj.s64, src, 2 * n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(adj.s64 + 4 * n3, src + 2 * n3, n3 * sizeof(double), cudaMemcpyDeviceToDevice, stream);
}

int Engine::backward(const float* dL_dx, const float* dL_dxo, float* dL_dk, float* dL_dscalar) {
    if (!adj.ready) return fail(VISG_ERR_STATE, "visg_backward needs a visg_forward first");
    if (!dL_dx) return fail(VISG_ERR_INVALID_ARG, "dL_dx is NULL");
    const size_t n3 = 3 * (size_t)N, st = 9 * (size_t)N;
    double* lam_in_x = adj.lam;
    double* lam_in_xo = adj.lam + n3;
    double* lam_out_x = adj.lam + 2 * n3;
    double* lam_out_xo = adj.lam + 3 * n3;
    std::vector<double> seed(2 * n3, 0.0);
    for (size_t k = 0; k < n3; ++k) seed[k] = dL_dx[k];
    if (dL_dxo)
        for (size_t k = 0; k < n3; ++k) seed[n3 + k] = dL_dxo[k];
    CU(cudaMemcpyAsync(lam_in_x, seed.data(), 2 * n3 * sizeof(double), cudaMemcpyHostToDevice, stream));
    CU(cudaMemsetAsync(adj.dk, 0, (size_t)std::max<int64_t>(E, 1) * sizeof(double), stream));
    CU(cudaMemsetAsync(adj.dsc, 0, 3 * sizeof(double), stream));
    AdjArgs a;
    a.rowp = d_rowp;
    a.ent = d_ent;
    a.kent = d_k;
    a.rev = adj.rev;
    a.G = adj.G;
    a.dk = adj.dk;
    a.dscalar = adj.dsc;
    a.n = (int)N;
    a.p = step_params();
    for (int seg = (int)adj.ck.size() - 1; seg >= 0; --seg) {
        const int s0 = seg * adj.ckpt, s1 = std::min(s0 + adj.ckpt, adj.nsteps);
        CU(load64(adj.ck[seg]));
        int c = 0;
        for (int t = s0; t < s1; ++t) {
            CU(save64(c, adj.rec + (size_t)(t - s0) * st));
            CU(step64(c));
            c ^= 1;
        }
        CU(save64(c, adj.rec + (size_t)(s1 - s0) * st));
        for (int t = s1 - 1; t >= s0; --t) {
            const double* r = adj.rec + (size_t)(t - s0) * st;
            a.x = r;
            a.xo = r + n3;
            a.n_in = r + 2 * n3;  // the normals entering step t
            a.n_out = adj.rec + (size_t)(t - s0 + 1) * st + 2 * n3;
            a.lx_in = lam_in_x;
            a.lxo_in = lam_in_xo;
            a.lx_out = lam_out_x;
            a.lxo_out = lam_out_xo;
            CU(launch_adjoint_step(a, stream));
            std::swap(lam_in_x, lam_out_x);
            std::swap(lam_in_xo, lam_out_xo);
        }
    }
    std::vector<double> dkm((size_t)std::max<int64_t>(E, 1));
    double dsc[3];
    CU(cudaMemcpyAsync(dkm.data(), adj.dk, (size_t)E * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CU(cudaMemcpyAsync(dsc, adj.dsc, sizeof dsc, cudaMemcpyDeviceToHost, stream));
    if (int r = sync()) return r;
    bool finite = std::isfinite((float)dsc[0]) && std::isfinite((float)dsc[1]) && std::isfinite((float)dsc[2]);
    for (int64_t c = 0; c < E && finite; ++c) finite = std::isfinite((float)dkm[c]);
    if (dL_dk)
        for (int64_t c = 0; c < E; ++c) dL_dk[merged_pos[c]] = (float)dkm[c];
    if (dL_dscalar)
        for (int k = 0; k < 3; ++k) dL_dscalar[k] = (float)dsc[k];
    if (!finite)
        return fail(VISG_ERR_DIVERGED,
                    "the gradient is not finite in float: the trajectory's sensitivity overflowed (an unstable "
                    "forward, or a long stretch of sustained contact at a step size where a projected vertex's "
                    "update amplifies perturbations); the values were written as computed");
    return VISG_OK;
}
