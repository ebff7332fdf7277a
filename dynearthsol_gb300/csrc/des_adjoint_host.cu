// des_adjoint_host.cu -- host side of the reverse mode: the window's
// forward with checkpoints, the per-segment recompute onto a tape of step
// records, and the reverse sweep (des_adjoint_forward/backward).
//
// Memory: a checkpoint holds the state and its derived fields (~180 B per
// tet); the tape of one segment holds checkpoint_every + 1 step records
// (~319 B per tet each, the forward values the reverse kernels read; the
// stress after NMD_stress is rebuilt from them).  At 1M tets and 50 steps
// per segment that is ~16 GB of HBM.
//
// The forward tapes the window's last segment itself: it writes each of
// its steps' records as it goes, so the backward, which reverses that
// segment first, recomputes only the others.  The tape is the one the
// backward needs anyway.  A window of one segment (checkpoint_every >=
// nsteps) is then taped whole, and its backward runs the reverse kernels
// alone: 500 steps of the 998,400-tet case are ~160 GB, which GB300's HBM
// holds.
#include <algorithm>
#include <vector>

#include "des_adjoint.cuh"
#include "des_ctx.cuh"
#include "des_kernels.cuh"

namespace des {

namespace {

size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// bump allocator over one device allocation
struct Carver {
    std::vector<std::pair<void **, size_t>> slots;
    void add(void **p, size_t bytes) { slots.push_back({p, al256(std::max<size_t>(bytes, 8))}); }
    size_t total() const
    {
        size_t t = 0;
        for (auto &s : slots) t += s.second;
        return t;
    }
    void assign(char *base)
    {
        size_t off = 0;
        for (auto &s : slots) {
            *s.first = base + off;
            off += s.second;
        }
    }
};

// the fields of a state and its derived fields, all [.][nn] / [.][ne] SoA
struct StateRef {
    double *x, *v, *T, *s, *pls, *volo, *vol, *shp, *mass, *tmass, *voln;
};

void add_state(Carver &cv, StateRef &r, size_t nn, size_t ne)
{
    const size_t D = sizeof(double);
    cv.add((void **)&r.x, 3 * nn * D);
    cv.add((void **)&r.v, 3 * nn * D);
    cv.add((void **)&r.T, nn * D);
    cv.add((void **)&r.s, 6 * ne * D);
    cv.add((void **)&r.pls, ne * D);
    cv.add((void **)&r.volo, ne * D);
    cv.add((void **)&r.vol, ne * D);
    cv.add((void **)&r.shp, 12 * ne * D);
    cv.add((void **)&r.mass, nn * D);
    cv.add((void **)&r.tmass, nn * D);
    cv.add((void **)&r.voln, nn * D);
}

StateRef live_state(const des_ctx *c)
{
    const KP &p = c->kp;
    return StateRef{p.x, p.v, p.T, p.stress, p.pls, p.vol_old, p.vol, p.shp, p.mass, p.tmass, p.vol_n};
}

StateRef tape_state(const TapeStep &t)
{
    return StateRef{t.x, t.v, t.T, t.s, t.pls, t.volo, t.vol, t.shp, t.mass, t.tmass, t.voln};
}

cudaError_t copy_state(const StateRef &dst, const StateRef &src, size_t nn, size_t ne, cudaStream_t s)
{
    const size_t D = sizeof(double);
    const std::pair<std::pair<double *, const double *>, size_t> f[] = {
        {{dst.x, src.x}, 3 * nn}, {{dst.v, src.v}, 3 * nn},     {{dst.T, src.T}, nn},
        {{dst.s, src.s}, 6 * ne}, {{dst.pls, src.pls}, ne},     {{dst.volo, src.volo}, ne},
        {{dst.vol, src.vol}, ne}, {{dst.shp, src.shp}, 12 * ne}, {{dst.mass, src.mass}, nn},
        {{dst.tmass, src.tmass}, nn}, {{dst.voln, src.voln}, nn}};
    for (auto &e : f) {
        cudaError_t r = cudaMemcpyAsync(e.first.first, e.first.second, e.second * D, cudaMemcpyDeviceToDevice, s);
        if (r != cudaSuccess) return r;
    }
    return cudaSuccess;
}

}  // namespace

struct AdjWork {
    char *buf_mem = nullptr;
    AdjBufs a{};
    int nblk_vbc = 0;
    char *tape_mem = nullptr;
    int cap = 0;
    std::vector<TapeStep> tape;
    char *ck_mem = nullptr;
    std::vector<StateRef> ck;
    char *final_pool = nullptr;
    int K = 0, C = 0, nseg = 0;
    double dt = 0;
    bool recorded = false;
    int tape_seg = -1;   // the segment whose records the tape holds (-1: none)
};

void adj_free(des_ctx *c)
{
    AdjWork *w = c->adj;
    if (!w) return;
    cudaFree(w->buf_mem);
    cudaFree(w->tape_mem);
    cudaFree(w->ck_mem);
    cudaFree(w->final_pool);
    delete w;
    c->adj = nullptr;
}

}  // namespace des

namespace des {
namespace {

#define CKA(call)                                               \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return ctx_cuda_fail(c, e_, #call); \
    } while (0)

// adjoint buffers and the element -> facet lists, once per context
int alloc_buffers(des_ctx *c, AdjWork *w)
{
    if (w->buf_mem) return DES_OK;
    const size_t nn = c->nn, ne = c->ne, nbf = std::max(c->nbf, 1), D = sizeof(double);
    AdjBufs &a = w->a;
    w->nblk_vbc = adj_vbc_blocks(c->kp);
    Carver cv;
    int *e2f_off, *e2f_ent;
    cv.add((void **)&a.ax, 3 * nn * D);
    cv.add((void **)&a.av, 3 * nn * D);
    cv.add((void **)&a.aT, nn * D);
    cv.add((void **)&a.as, 6 * ne * D);
    cv.add((void **)&a.apls, ne * D);
    cv.add((void **)&a.avolo, ne * D);
    cv.add((void **)&a.avol, ne * D);
    cv.add((void **)&a.ashp, 12 * ne * D);
    cv.add((void **)&a.am, nn * D);
    cv.add((void **)&a.atm, nn * D);
    cv.add((void **)&a.avn, nn * D);
    cv.add((void **)&a.af, 3 * nn * D);
    cv.add((void **)&a.antmp, nn * D);
    cv.add((void **)&a.adpn, nn * D);
    cv.add((void **)&a.atdot, nn * D);
    cv.add((void **)&a.aedot, 6 * ne * D);
    cv.add((void **)&a.aedv, ne * D);
    cv.add((void **)&a.adp, ne * D);
    cv.add((void **)&a.arho, ne * D);
    cv.add((void **)&a.slot3, 12 * ne * D);
    cv.add((void **)&a.slotx, 12 * ne * D);
    cv.add((void **)&a.slot1, 4 * ne * D);
    cv.add((void **)&a.fslot, 9 * nbf * D);
    cv.add((void **)&a.frho, nbf * D);
    cv.add((void **)&a.g, (size_t)DES_EF_COUNT * ne * D);
    cv.add((void **)&a.gvbc, (size_t)w->nblk_vbc * DES_NBDRYTYPES * D);
    cv.add((void **)&e2f_off, (ne + 1) * sizeof(int));
    cv.add((void **)&e2f_ent, nbf * sizeof(int));
    cudaError_t e = cudaMalloc((void **)&w->buf_mem, cv.total());
    if (e != cudaSuccess) {
        (void)cudaGetLastError();   // reported here, not at the next launch check
        return ctx_fail(c, DES_ENOMEM, "adjoint buffers: cudaMalloc(%zu bytes): %s", cv.total(), cudaGetErrorString(e));
    }
    cv.assign(w->buf_mem);
    a.e2f_off = e2f_off;
    a.e2f_ent = e2f_ent;
    // element -> boundary facets, ascending facet id
    std::vector<int> fe(c->nbf), off(ne + 1, 0), ent(std::max(c->nbf, 1), 0);
    if (c->nbf > 0) CKA(cudaMemcpy(fe.data(), c->kp.fac_elem, c->nbf * sizeof(int), cudaMemcpyDeviceToHost));
    for (int q = 0; q < c->nbf; ++q) off[fe[q] + 1]++;
    for (size_t e2 = 0; e2 < ne; ++e2) off[e2 + 1] += off[e2];
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int q = 0; q < c->nbf; ++q) ent[fill[fe[q]]++] = q;
    CKA(cudaMemcpy(e2f_off, off.data(), (ne + 1) * sizeof(int), cudaMemcpyHostToDevice));
    CKA(cudaMemcpy(e2f_ent, ent.data(), ent.size() * sizeof(int), cudaMemcpyHostToDevice));
    return DES_OK;
}

void add_tape_step(Carver &cv, TapeStep &t, size_t nn, size_t ne)
{
    const size_t D = sizeof(double);
    cv.add((void **)&t.x, 3 * nn * D);
    cv.add((void **)&t.v, 3 * nn * D);
    cv.add((void **)&t.T, nn * D);
    cv.add((void **)&t.s, 6 * ne * D);
    cv.add((void **)&t.pls, ne * D);
    cv.add((void **)&t.volo, ne * D);
    cv.add((void **)&t.vol, ne * D);
    cv.add((void **)&t.shp, 12 * ne * D);
    cv.add((void **)&t.mass, nn * D);
    cv.add((void **)&t.tmass, nn * D);
    cv.add((void **)&t.voln, nn * D);
    cv.add((void **)&t.edot, 6 * ne * D);
    cv.add((void **)&t.tdot, nn * D);
    cv.add((void **)&t.ntmp, nn * D);
    cv.add((void **)&t.edv, ne * D);
    cv.add((void **)&t.sstar, 6 * ne * D);
    cv.add((void **)&t.dp, ne * D);
    cv.add((void **)&t.rho, ne * D);
    cv.add((void **)&t.dpn, nn * D);
    cv.add((void **)&t.f, 3 * nn * D);
    cv.add((void **)&t.visc, ne * D);
    cv.add((void **)&t.evp, ne);
}

int alloc_tape(des_ctx *c, AdjWork *w, int cap)
{
    if (w->tape_mem && w->cap == cap) return DES_OK;
    cudaFree(w->tape_mem);
    w->tape_mem = nullptr;
    w->cap = 0;
    w->tape_seg = -1;
    w->tape.clear();
    const size_t nn = c->nn, ne = c->ne;
    // the whole tape against the free device memory, before any allocation
    // (the host records too are sized by cap)
    TapeStep probe{};
    Carver one;
    add_tape_step(one, probe, nn, ne);
    const size_t need = one.total() * ((size_t)cap + 1);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && need > free_b)
        return ctx_fail(c, DES_ENOMEM, "adjoint tape of %d steps: %zu bytes, %zu free on the device", cap, need,
                        free_b);
    w->tape.assign((size_t)cap + 1, TapeStep{});
    Carver cv2;
    for (auto &t : w->tape) add_tape_step(cv2, t, nn, ne);
    cudaError_t e = cudaMalloc((void **)&w->tape_mem, cv2.total());
    if (e != cudaSuccess) {
        (void)cudaGetLastError();   // reported here, not at the next launch check
        w->tape.clear();
        return ctx_fail(c, DES_ENOMEM, "adjoint tape of %d steps: cudaMalloc(%zu bytes): %s", cap, cv2.total(),
                        cudaGetErrorString(e));
    }
    cv2.assign(w->tape_mem);
    w->cap = cap;
    return DES_OK;
}

// one FP64 step with dt held (the fused step's kernels without compute_dt);
// with a tape record, the start state and the forward values the reverse
// kernels read are copied into it
int adj_step(des_ctx *c, const TapeStep *t)
{
    KP p = ctx_step_kp(c);
    if (t) {   // the rheology writes the viscosity and the EVP branch it took
        p.tape_visc = t->visc;
        p.tape_evp = t->evp;
    }
    cudaStream_t s = c->stream;
    const size_t nn = c->nn, ne = c->ne, D = sizeof(double);
    auto cp = [&](double *dst, const double *src, size_t n) {
        return cudaMemcpyAsync(dst, src, n * D, cudaMemcpyDeviceToDevice, s);
    };
    int n = 0;
    if (t) CKA(copy_state(tape_state(*t), live_state(c), nn, ne, s));
    // strain rate, heat and dvoldt as the fused FP64 step forms them
    const bool thermal = p.prm.has_thermal_diffusion != 0;
    n += launch_elem_pass(p, s, thermal);
    if (t) CKA(cp(t->edot, p.srate, 6 * ne));
    n += launch_node_pass(p, s, thermal);
    if (t) {
        if (thermal) CKA(cp(t->tdot, p.tdot, nn));
        CKA(cp(t->ntmp, p.ntmp, nn));
    }
    n += launch_update_stress(p, s, true);
    if (t) {
        CKA(cp(t->sstar, p.stress, 6 * ne));
        CKA(cp(t->dp, p.dp, ne));
        CKA(cp(t->rho, p.rho_e, ne));
        CKA(cp(t->edv, p.edvoldt, ne));
    }
    n += launch_nmd_gather(p, s);
    if (t) CKA(cp(t->dpn, p.ntmp, nn));
    n += launch_nmd_correct(p, s, true);
    n += launch_force(p, s, true);
    if (t) CKA(cp(t->f, p.f, 3 * nn));
    // mass from the geometry pass's element terms: the same sums, in the same
    // order, as compute_mass's node gather (launch_mass), at a fifth of its cost
    int geo = GEO_COPY_OLD | GEO_VOLUME | GEO_SHAPE | GEO_MASS_TERMS;
    if (p.mat.rheol_type & DES_RH_ELASTIC) geo |= GEO_ROTATE;
    n += launch_geometry(p, s, geo);
    n += launch_mass_sum(p, s);
    return ctx_check_launch(c, n);
}

int adj_reverse_step(des_ctx *c, AdjWork *w, const TapeStep &t, const TapeStep &t1)
{
    const KP p = ctx_step_kp(c);
    cudaStream_t s = c->stream;
    const AdjBufs &a = w->a;
    int n = 0;
    n += launch_adj_end_geometry(p, a, t, t1, w->dt, s);
    n += launch_adj_motion(p, a, t, t1, w->dt, s);
    n += launch_adj_force(p, a, t, s);
    n += launch_adj_nmd_nodes(p, a, t, s);
    n += launch_adj_stress(p, a, t, t1, w->dt, s);
    n += launch_adj_nodes_heat(p, a, t, t1, w->dt, s);
    n += launch_adj_kinematics(p, a, t, s);
    n += launch_adj_gather_vT(p, a, s);
    return ctx_check_launch(c, n);
}

int check_supported(des_ctx *c)
{
    const KP &p = c->kp;
    if (c->nd != 3) return ctx_fail(c, DES_EINPUT, "adjoint: 3D only");
    if (c->precision != DES_PREC_FP64) return ctx_fail(c, DES_EINPUT, "adjoint: FP64 contexts only");
    if (p.mat.nmat != 1 || p.emark) return ctx_fail(c, DES_EINPUT, "adjoint: one material without markers only");
    if (p.mat.rheol_type == DES_RH_VISCOUS) return ctx_fail(c, DES_EINPUT, "adjoint: viscous rheology unsupported");
    if (p.mat.is_plane_strain) return ctx_fail(c, DES_EINPUT, "adjoint: plane strain unsupported");
    if (!c->has_state) return ctx_fail(c, DES_EINPUT, "adjoint: no state uploaded");
    return DES_OK;
}

}  // namespace

}  // namespace des

using namespace des;

int des_adjoint_forward(des_ctx *c, int nsteps, int checkpoint_every)
{
    if (!c || nsteps < 1 || checkpoint_every < 1) return DES_EINPUT;
    int rc = check_supported(c);
    if (rc) return rc;
    if (!c->adj) c->adj = new AdjWork;
    AdjWork *w = c->adj;
    w->recorded = false;
    if ((rc = alloc_buffers(c, w))) return rc;
    const size_t nn = c->nn, ne = c->ne;
    const int C = std::min(checkpoint_every, nsteps);
    const int nseg = (nsteps + C - 1) / C, last0 = (nseg - 1) * C;
    w->tape_seg = -1;
    if ((rc = alloc_tape(c, w, C))) return rc;
    if ((int)w->ck.size() != nseg) {
        cudaFree(w->ck_mem);
        w->ck_mem = nullptr;
        w->ck.assign(nseg, StateRef{});
        Carver cv;
        for (auto &r : w->ck) add_state(cv, r, nn, ne);
        cudaError_t e = cudaMalloc((void **)&w->ck_mem, cv.total());
        if (e != cudaSuccess) {
            w->ck.clear();
            (void)cudaGetLastError();   // reported here, not at the next launch check
            return ctx_fail(c, DES_ENOMEM, "adjoint checkpoints: cudaMalloc(%zu bytes): %s", cv.total(),
                            cudaGetErrorString(e));
        }
        cv.assign(w->ck_mem);
    }
    if (!w->final_pool) CKA(cudaMalloc((void **)&w->final_pool, c->pool_bytes));
    Clock clk;
    CKA(cudaMemcpyAsync(&clk, c->kp.clk, sizeof(Clock), cudaMemcpyDeviceToHost, c->stream));
    CKA(cudaStreamSynchronize(c->stream));
    w->dt = clk.dt;
    for (int k = 0; k < nsteps; ++k) {
        if (k % C == 0) CKA(copy_state(w->ck[k / C], live_state(c), nn, ne, c->stream));
        if ((rc = adj_step(c, k >= last0 ? &w->tape[k - last0] : nullptr))) return rc;
    }
    CKA(copy_state(tape_state(w->tape[nsteps - last0]), live_state(c), nn, ne, c->stream));
    CKA(cudaMemcpyAsync(w->final_pool, c->pool, c->pool_bytes, cudaMemcpyDeviceToDevice, c->stream));
    w->K = nsteps;
    w->C = C;
    w->nseg = nseg;
    w->tape_seg = nseg - 1;
    w->recorded = true;
    return DES_OK;
}

int des_adjoint_backward(des_ctx *c, const des_host_state *seed, des_host_state *start_adjoint,
                         des_adjoint_grad *grad)
{
    if (!c) return DES_EINPUT;
    AdjWork *w = c->adj;
    if (!w || !w->recorded) return ctx_fail(c, DES_EINPUT, "des_adjoint_backward before des_adjoint_forward");
    int rc = alloc_tape(c, w, w->C);
    if (rc) return rc;
    const size_t nn = c->nn, ne = c->ne;
    const AdjBufs &a = w->a;
    cudaStream_t s = c->stream;
    CKA(cudaMemsetAsync(w->buf_mem, 0, (char *)a.e2f_off - w->buf_mem, s));
    if (seed) {
        if (seed->coord && (rc = ctx_put_field(c, seed->coord, a.ax, c->nn, 3))) return rc;
        if (seed->vel && (rc = ctx_put_field(c, seed->vel, a.av, c->nn, 3))) return rc;
        if (seed->temperature && (rc = ctx_put_field(c, seed->temperature, a.aT, c->nn, 1))) return rc;
        if (seed->stress && (rc = ctx_put_field(c, seed->stress, a.as, c->ne, 6))) return rc;
        if (seed->plstrain && (rc = ctx_put_field(c, seed->plstrain, a.apls, c->ne, 1))) return rc;
        // the final volume_old is the volume at the last step's start: its
        // adjoint enters that step's reverse as the next state's avolo
        if (seed->volume_old && (rc = ctx_put_field(c, seed->volume_old, a.avolo, c->ne, 1))) return rc;
    }
    for (int seg = w->nseg - 1; seg >= 0; --seg) {
        const int k0 = seg * w->C, L = std::min(w->C, w->K - k0);
        if (w->tape_seg != seg) {   // recompute the segment from its checkpoint onto the tape
            w->tape_seg = -1;
            CKA(copy_state(live_state(c), w->ck[seg], nn, ne, s));
            for (int j = 0; j < L; ++j)
                if ((rc = adj_step(c, &w->tape[j]))) return rc;
            CKA(copy_state(tape_state(w->tape[L]), live_state(c), nn, ne, s));
            w->tape_seg = seg;
        }
        for (int j = L - 1; j >= 0; --j)
            if ((rc = adj_reverse_step(c, w, w->tape[j], w->tape[j + 1]))) return rc;
    }
    {
        const KP p = ctx_step_kp(c);
        rc = ctx_check_launch(c, launch_adj_start_geometry(p, a, w->tape[0], s) + launch_adj_gather_xT(p, a, s));
        if (rc) return rc;
    }
    if (grad) {
        for (int k = 0; k < DES_EF_COUNT; ++k)
            if (grad->elem[k])
                CKA(cudaMemcpyAsync(grad->elem[k], a.g + (size_t)k * ne, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
        std::vector<double> part((size_t)w->nblk_vbc * DES_NBDRYTYPES);
        CKA(cudaMemcpyAsync(part.data(), a.gvbc, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        CKA(cudaStreamSynchronize(s));
        for (int ib = 0; ib < DES_NBDRYTYPES; ++ib) {
            double acc = 0;
            for (int b = 0; b < w->nblk_vbc; ++b) acc += part[(size_t)b * DES_NBDRYTYPES + ib];
            grad->vbc_values[ib] = acc;
        }
    }
    if (start_adjoint) {
        if (start_adjoint->coord && (rc = ctx_get_field(c, a.ax, start_adjoint->coord, c->nn, 3))) return rc;
        if (start_adjoint->vel && (rc = ctx_get_field(c, a.av, start_adjoint->vel, c->nn, 3))) return rc;
        if (start_adjoint->temperature && (rc = ctx_get_field(c, a.aT, start_adjoint->temperature, c->nn, 1)))
            return rc;
        if (start_adjoint->stress && (rc = ctx_get_field(c, a.as, start_adjoint->stress, c->ne, 6))) return rc;
        if (start_adjoint->plstrain && (rc = ctx_get_field(c, a.apls, start_adjoint->plstrain, c->ne, 1)))
            return rc;
        if (start_adjoint->volume_old && (rc = ctx_get_field(c, a.avolo, start_adjoint->volume_old, c->ne, 1)))
            return rc;
    }
    CKA(cudaMemcpyAsync(c->pool, w->final_pool, c->pool_bytes, cudaMemcpyDeviceToDevice, s));
    CKA(cudaStreamSynchronize(s));
    return DES_OK;
}
