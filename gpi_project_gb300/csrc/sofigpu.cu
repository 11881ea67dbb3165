// sofigpu.cu -- C ABI of the GB300 time-stepping library (see include/sofigpu.h).
//
// A context owns, on one device and one CUDA stream, the wavefields of
// `nshots` resident shots, the prepared model (shared or per shot), the CPML
// memory, the acquisition and the sections. sofi_run() issues the kernels of
// sofi_kernels.cuh in the reference's phase order for each time step.
#include "sofigpu.h"
#include "sofi_kernels.cuh"
#include "sofi_launch.h"
#include "sofi_dispatch.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <vector>

using namespace sofi;

namespace {

constexpr int kGraphSteps = 32;

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? SOFI_E_NOMEM : SOFI_E_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                        \
    } while (0)

// Holberg / Taylor operator coefficients (reference holbergcoeff.c:40-82; the
// published tables: Taylor row, then Holberg 1987 for 0.1%, 0.5%, 1%, 3%).
const double kHolberg[5][6][7] = {
    {{23.0, 1.0, 0, 0, 0, 0, 0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0, 0, 0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0, 0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0, 35.0 / 294912.0, 0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0, -5445.0 / 1835008.0,
      847.0 / 2359296.0, -63.0 / 2883584.0}},
    {{49.7, 1.0010, 0, 0, 0, 0, 0},
     {8.32, 1.1382, -0.046414, 0, 0, 0, 0},
     {4.77, 1.1965, -0.078804, 0.0081781, 0, 0, 0},
     {3.69, 1.2257, -0.099537, 0.018063, -0.0026274, 0, 0},
     {3.19, 1.2415, -0.11231, 0.026191, -0.0064682, 0.001191, 0},
     {2.91, 1.2508, -0.12034, 0.032131, -0.010142, 0.0029857, -0.00066667}},
    {{22.2, 1.0050, 0, 0, 0, 0, 0},
     {5.65, 1.1534, -0.052806, 0, 0, 0, 0},
     {3.74, 1.2111, -0.088313, 0.011768, 0, 0, 0},
     {3.11, 1.2367, -0.10815, 0.023113, -0.0046905, 0, 0},
     {2.80, 1.2496, -0.11921, 0.031130, -0.0093272, 0.0025161, 0},
     {2.62, 1.2568, -0.12573, 0.036423, -0.013132, 0.0047484, -0.0015979}},
    {{15.8, 1.0100, 0, 0, 0, 0, 0},
     {4.80, 1.1640, -0.057991, 0, 0, 0, 0},
     {3.39, 1.2192, -0.094070, 0.014608, 0, 0, 0},
     {2.90, 1.2422, -0.11269, 0.026140, -0.0064054, 0, 0},
     {2.65, 1.2534, -0.12257, 0.033755, -0.011081, 0.0036784, 0},
     {2.51, 1.2596, -0.12825, 0.038550, -0.014763, 0.0058619, -0.0024538}},
    {{9.16, 1.0300, 0, 0, 0, 0, 0},
     {3.47, 1.1876, -0.072518, 0, 0, 0, 0},
     {2.91, 1.2341, -0.10569, 0.022589, 0, 0, 0},
     {2.61, 1.2516, -0.12085, 0.032236, -0.011459, 0, 0},
     {2.45, 1.2596, -0.12829, 0.038533, -0.014681, 0.0072580, 0},
     {2.36, 1.2640, -0.13239, 0.042217, -0.017803, 0.0081959, -0.0051848}},
};

bool is_visco(int weq) { return weq == SOFI_VEL_ISO || weq == SOFI_VEL_VTI || weq == SOFI_VEL_TTI; }
int kind_of(int weq)
{
    if (weq == SOFI_AC_ISO)
        return AC;
    return (weq == SOFI_EL_ISO || weq == SOFI_VEL_ISO) ? ISO : (weq <= SOFI_VEL_VTI ? VTI : TTI);
}

struct FieldSlot {
    const char *name;   // ABI name
    const char *alt;    // accepted alias (e.g. unrelaxed name for viscoelastic media)
    size_t off;         // offset of the const float* in Model
};

#define SLOT(n, a, m) {n, a, offsetof(Model, m)}
const FieldSlot kSlots[] = {
    SLOT("prip", nullptr, prip), SLOT("prjp", nullptr, prjp), SLOT("g", nullptr, g), SLOT("f", nullptr, f),
    SLOT("fipjp", nullptr, fipjp), SLOT("d_base", nullptr, db), SLOT("e_base", nullptr, eb),
    SLOT("dip_base", nullptr, dipb), SLOT("c11", "c11u", c11), SLOT("c13", "c13u", c13),
    SLOT("c33", "c33u", c33), SLOT("c15", "c15u", c15), SLOT("c35", "c35u", c35),
    SLOT("c55ipjp", "c55ipjpu", c55ipjp), SLOT("c15ipjp", "c15ipjpu", c15ipjp),
    SLOT("c35ipjp", "c35ipjpu", c35ipjp), SLOT("c11d_base", nullptr, c11b), SLOT("c13d_base", nullptr, c13b),
    SLOT("c33d_base", nullptr, c33b), SLOT("c15d_base", nullptr, c15b), SLOT("c35d_base", nullptr, c35b),
    SLOT("c55ipjpd_base", nullptr, c55ipjpb), SLOT("c15ipjpd_base", nullptr, c15ipjpb),
    SLOT("c35ipjpd_base", nullptr, c35ipjpb), SLOT("ppi", nullptr, ppi), SLOT("pu", nullptr, pu),
    SLOT("taus", nullptr, taus), SLOT("taup", nullptr, taup), SLOT("absorb", nullptr, absorb),
};
#undef SLOT

const char *kVectors[12] = {"K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half",
                            "K_y", "a_y", "b_y", "K_y_half", "a_y_half", "b_y_half"};

// which model slots a wave equation reads
std::vector<std::string> needed_fields(const sofi_config &c)
{
    int k = kind_of(c.weq);
    bool visco = is_visco(c.weq);
    if (k == AC) {
        // initmem_model.c:33-39: the acoustic model has no mu
        std::vector<std::string> a = {"prip", "prjp", "g"};
        if (c.fw > 0 && c.abs_type == 2)
            a.push_back("absorb");
        return a;
    }
    std::vector<std::string> v = {"prip", "prjp", "ppi", "pu"};
    if (k == ISO) {
        v.insert(v.end(), {"g", "f", "fipjp"});
        if (visco) {
            v.insert(v.end(), {"d_base", "e_base", "dip_base"});
            if (c.free_surf)
                v.insert(v.end(), {"taus", "taup"});
        }
    } else {
        v.insert(v.end(), {"c11", "c13", "c33", "c55ipjp"});
        if (k == TTI)
            v.insert(v.end(), {"c15", "c35", "c15ipjp", "c35ipjp"});
        if (visco) {
            v.insert(v.end(), {"c11d_base", "c13d_base", "c33d_base", "c55ipjpd_base"});
            if (k == TTI)
                v.insert(v.end(), {"c15d_base", "c35d_base", "c15ipjpd_base", "c35ipjpd_base"});
        }
    }
    if (c.fw > 0 && c.abs_type == 2)
        v.push_back("absorb");
    return v;
}

struct ShotAcq {
    std::vector<int> ix, iy, type;
    std::vector<float> amp, sn, cs, sn2, cs2, sig;
    std::vector<int> rix, riy;
};

int pitch_for(int nx) { return ((nx + 2 * HX + 31) / 32) * 32; }

}  // namespace

struct sofi_ctx {
    sofi_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Geo G{};
    Wave W{};
    Model M{};
    Acq A{};
    int nmodels = 1;
    int nd = 2;
    std::vector<void *> allocs;
    std::vector<ShotAcq> acq;
    bool acq_dirty = true;
    bool has_force = false;
    int total_src = 0, total_rec = 0;
    void *acq_buf = nullptr;
    float *d_sec = nullptr;
    unsigned char *d_cellflag = nullptr;  // Acq::cell_flag
    int *d_status = nullptr;
    int step = 0;
    float last_ms = 0.f;
    bool run_pending = false;  // ev0/ev1 recorded by a sofi_run not yet synchronised
    int vw = 4;                // velocity kernel: cells per thread in x (4 or 2), 0 = vrows rows per thread
    int vrows = 1;             // rows per thread of the one-cell velocity kernel (1, 2 or 4)
    int fwi_vw = 4, fwi_sw = 4; // an FWI pass's forward steps: cells per thread of the FWI kernels
    bool tuning = false;       // the autotuner's launches are being issued (plain kernels only)
    // FWI gradient pass of one shot (sofi_fwi_*; sofi_fwi.cu)
    bool fwi = false;          // the forward runs store the gradient quantities
    bool fwi_back = false;     // the backward run is being issued
    FwiDev F{};
    int *d_noacq = nullptr;    // two zero ints: the backward run's empty source list
    size_t fwi_cells_cap = 0;  // capacity of the receiver-cell arrays
    // checkpointed pass (the store does not hold NT steps): the state after
    // steps K, 2K, ... of the forward run; every segment is recomputed into a
    // K-slot store before its backward steps
    int fwi_K = 0;             // 0: the forward run is stored whole
    int fwi_nseg = 1;
    size_t fwi_state = 0;      // floats of one state (wavefield and CPML memory)
    size_t fwi_slots = 0;      // slots the store holds
    float *fwi_ckpt = nullptr; // [nseg - 1][fwi_state]
    size_t fwi_ckpt_cap = 0;
    float *fwi_tmp = nullptr;  // the backward state while a segment is recomputed
    bool fwi_store_on = true;  // k_fwi_store runs (off in the checkpointing forward run)
    bool fwi_nosnap = false;   // a recomputed segment takes no snapshots
    int *d_fwi_base = nullptr; // device: FwiDev::base
    int sw = 0;                // ISO / VTI stress kernel: cells per thread in x (4 or 2), 0 = one
    bool vnarrow = false;      // four-cell velocity / stress kernels on 8 x 32-thread blocks
    bool snarrow = false;      //   (narrow_v_applies / narrow_s_applies)
    bool sw_fixed = false;     // SOFI_SW chose it
    bool tuned = false;        // autotuner ran (or was skipped) for this context
    bool tune_fixed = false;   // SOFI_VROWS chose the variant
    bool pristine = false;     // every state array zero: reset(-1) and no set_field since
    // CUDA graph of kGraphSteps time steps, replayed for every chunk without
    // snapshot or timed steps (the step number lives in G.step_ctr)
    bool use_graph = true;
    bool pdl = true;  // programmatic dependent launch of the step kernels (launch_pdl)
    bool graph_dirty = true;
    cudaGraphExec_t graph_exec = nullptr;   // the step graph
    bool graph_ok = false;
    long long graph_launches = 0;  // kernels per replay
    bool postf = true;         // k_post's work inside the one-cell stress kernel where it applies (SOFI_POSTF=0: off)
    bool tti_split = false;    // TTI: derivative fields through HBM (two kernels) instead of fused
    bool tti_fused = false;    // TTI: the one-pass kernel on 32 x 8 tiles everywhere (no four-cell interior tiles)
    // snapshots
    int snap_nx = 0, snap_ny = 0, snap_total = 0, nsnap = 0;
    float *d_snap = nullptr;
    // instrumentation
    long long launches = 0;
    int time_every = 0;
    std::vector<cudaEvent_t> tev;   // 3 events per timed step: before v, after v, after s
    size_t tev_used = 0;
    double t_v_ms = 0, t_s_ms = 0;
    long long t_count = 0;
    // completion events of the sofi_run calls still in flight (oldest first)
    std::deque<cudaEvent_t> run_ev;
    std::vector<cudaEvent_t> ev_free;
};

static void drop_graphs(sofi_ctx *c)
{
    if (c->graph_exec) {
        cudaGraphExecDestroy(c->graph_exec);
        c->graph_exec = nullptr;
    }
    c->graph_ok = false;
}

namespace {

int dalloc(sofi_ctx *c, void **p, size_t bytes)
{
    if (bytes == 0)
        bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, c->stream);
    if (e != cudaSuccess)
        return fail(SOFI_E_NOMEM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    c->allocs.push_back(*p);
    e = cudaMemsetAsync(*p, 0, bytes, c->stream);
    if (e != cudaSuccess)
        return fail(SOFI_E_CUDA, "memset: %s", cudaGetErrorString(e));
    return 0;
}

const float **slot_ptr(Model &M, const char *name, bool visco)
{
    for (const auto &s : kSlots) {
        if (!strcmp(s.name, name) || (s.alt && !strcmp(s.alt, name) && visco))
            return reinterpret_cast<const float **>(reinterpret_cast<char *>(&M) + s.off);
    }
    return nullptr;
}

int count_snapshots(const sofi_config &c)
{
    if (!c.snap)
        return 0;
    int n = 0;
    for (int nt = c.snap_first; nt <= c.snap_last && nt <= c.nt && nt >= 1; nt += (c.snap_inc > 0 ? c.snap_inc : c.nt + 1))
        n++;
    return n;
}

// Where upload_acq builds the per-cell flags that let the one-cell ISO / VTI
// stress kernel do the post work (post_fused): no free surface, 2nd-order
// time, and grids small enough (all shots) that a saved launch matters.
bool post_flags_apply(const sofi_config &c)
{
    const int kind = kind_of(c.weq);
    return (kind == ISO || kind == VTI) && !c.free_surf && c.fdorder_time != 4 &&
           (long long)c.nx * c.ny * c.nshots <= (4LL << 20);
}

long long fields_bytes(const sofi_config &c)
{
    long long pitch = pitch_for(c.nx), fsz = pitch * (c.ny + 2 * HY);
    // TTI: the fused stress kernel doubles the velocity-derivative CPML memory;
    // the two-kernel form (SOFI_TTI=split) holds 8 derivative fields instead
    const char *e = getenv("SOFI_TTI");
    const bool tti = kind_of(c.weq) == TTI, split = tti && e && strcmp(e, "split") == 0;
    // acoustic: sxx and syy are one array
    // FDORDER_TIME = 4: 24 history fields, memory variables in four levels
    const int ab = c.fdorder_time == 4;
    long long per_shot = (c.weq == SOFI_AC_ISO ? 4 : 5) + 3LL * (is_visco(c.weq) ? c.L : 0) * (ab ? 4 : 1) +
                         (split ? 8 : 0) + (ab ? 24 : 0);
    long long fw2 = 2LL * c.fw;
    long long psi = (c.abs_type == 1 && c.fw > 0) ? (tti && !split ? 6 : 4) * ((long long)c.ny * fw2 + fw2 * c.nx) : 0;
    long long nmod = c.shared_model ? 1 : c.nshots;
    long long nfields = (long long)needed_fields(c).size();
    long long bytes = 4 * (fsz * per_shot * c.nshots + psi * c.nshots + fsz * nfields * nmod);
    if (post_flags_apply(c))  // the per-cell flags of the post work (upload_acq)
        bytes += (long long)c.nx * c.ny * c.nshots;
    int nsnap = count_snapshots(c);
    if (nsnap) {
        long long sx = (c.nx - 1) / c.idx + 1, sy = (c.ny - 1) / c.idy + 1;
        bytes += 4LL * sx * sy * 5 * nsnap * c.nshots;
    }
    return bytes;
}

int check_config(const sofi_config *c)
{
    if (!c)
        return fail(SOFI_E_ARG, "null config");
    if (c->weq < SOFI_AC_ISO || c->weq == 1 || c->weq > SOFI_VEL_TTI)
        return fail(SOFI_E_ARG, "unsupported WEQ %d (AC_ISO = 0, EL_ISO..VEL_TTI = 2..7)", c->weq);
    // the reference allocates neither mu nor sxy for acoustic media
    // (initmem_model.c:33-39, initmem_wavefield.c:32-39): its free surface and
    // div/curl outputs would read them
    if (c->fdorder_time != 0 && c->fdorder_time != 2 && c->fdorder_time != 4)
        return fail(SOFI_E_ARG, "FDORDER_TIME must be 2 or 4 (got %d)", c->fdorder_time);
    // prepmod.c:160-186: 4th order in time exists for EL_ISO and VEL_ISO only
    if (c->fdorder_time == 4 && ((c->weq != SOFI_EL_ISO && c->weq != SOFI_VEL_ISO) || c->free_surf))
        return fail(SOFI_E_ARG, "FDORDER_TIME=4: EL_ISO or VEL_ISO without free surface only");
    if (c->weq == SOFI_AC_ISO && (c->free_surf || c->seismo >= 3 || c->snap >= 3))
        return fail(SOFI_E_ARG, "acoustic media: no free surface and no div/curl (SEISMO, SNAP <= 2)");
    if (c->fdorder < 2 || c->fdorder > 12 || (c->fdorder & 1))
        return fail(SOFI_E_ARG, "FDORDER must be 2,4,..,12 (got %d)", c->fdorder);
    if (c->maxrelerror < 0 || c->maxrelerror > 4)
        return fail(SOFI_E_ARG, "MAXRELERROR must be 0..4");
    int nd = c->fdorder / 2;
    if (c->nx < 2 * nd + 2 || c->ny < 2 * nd + 2)
        return fail(SOFI_E_ARG, "grid %dx%d too small for FDORDER %d", c->nx, c->ny, c->fdorder);
    if (c->nt < 1 || c->nshots < 1 || c->dt <= 0.f || c->dh <= 0.f)
        return fail(SOFI_E_ARG, "NT, nshots, DT and DH must be positive");
    if (is_visco(c->weq) && (c->L < 1 || c->L > MAXL))
        return fail(SOFI_E_ARG, "viscoelastic media need 1 <= L <= %d", MAXL);
    if (c->fw < 0 || 2 * c->fw > c->nx || 2 * c->fw > c->ny)
        return fail(SOFI_E_ARG, "frame width FW=%d does not fit the grid", c->fw);
    if (c->fw > 0 && c->abs_type != 1 && c->abs_type != 2)
        return fail(SOFI_E_ARG, "ABS_TYPE must be 1 (CPML) or 2 (damping)");
    if (c->abs_type == 2 && c->fw == 1)
        return fail(SOFI_E_ARG, "damping frame needs FW >= 2");
    if (c->free_surf && is_visco(c->weq) && kind_of(c->weq) != ISO)
        return fail(SOFI_E_ARG, "free surface is not defined for viscoelastic VTI/TTI media");
    if (c->seismo < 0 || c->seismo > 4 || c->snap < 0 || c->snap > 4)
        return fail(SOFI_E_ARG, "SEISMO and SNAP must be 0..4");
    if (c->seismo && c->ndt < 1)
        return fail(SOFI_E_ARG, "NDT must be >= 1");
    if (c->snap && (c->idx < 1 || c->idy < 1))
        return fail(SOFI_E_ARG, "IDX and IDY must be >= 1");
    return 0;
}

int upload_acq(sofi_ctx *c)
{
    // flatten per-shot sources / receivers into one device block
    int S = c->cfg.nshots, NT = c->cfg.nt;
    std::vector<int> soff(S + 1, 0), roff(S + 1, 0), last(S, 0);
    for (int s = 0; s < S; s++) {
        soff[s + 1] = soff[s] + (int)c->acq[s].ix.size();
        roff[s + 1] = roff[s] + (int)c->acq[s].rix.size();
        last[s] = c->acq[s].type.empty() ? 0 : c->acq[s].type.back();
    }
    int ns_src = soff[S], nrec = roff[S];
    c->has_force = false;
    // receivers grouped by (shot, column): the post-stress kernel samples the
    // receivers of its own column
    std::vector<int> colcnt((size_t)S * (c->cfg.nx + 1), 0), colidx(nrec > 0 ? nrec : 1, 0);
    for (int s = 0; s < S; s++)
        for (int k = roff[s]; k < roff[s + 1]; k++)
            colcnt[(size_t)s * (c->cfg.nx + 1) + c->acq[s].rix[k - roff[s]]]++;
    for (int s = 0; s < S; s++) {  // counts -> start of each column's group
        int *cc = &colcnt[(size_t)s * (c->cfg.nx + 1)];
        int run = roff[s];
        for (int i = 0; i <= c->cfg.nx; i++) {
            int n = cc[i];
            cc[i] = run;
            run += n;
        }
    }
    // colidx: receivers in column order; coloff[s][i-1] .. coloff[s][i] spans column i
    {
        std::vector<int> fill(colcnt);
        for (int s = 0; s < S; s++)
            for (int k = roff[s]; k < roff[s + 1]; k++) {
                int x = c->acq[s].rix[k - roff[s]];
                colidx[fill[(size_t)s * (c->cfg.nx + 1) + x]++] = k;
            }
    }
    std::vector<int> coloff((size_t)S * (c->cfg.nx + 1));
    for (int s = 0; s < S; s++)
        for (int i = 0; i <= c->cfg.nx; i++)
            coloff[(size_t)s * (c->cfg.nx + 1) + i] =
                (i < c->cfg.nx) ? colcnt[(size_t)s * (c->cfg.nx + 1) + i + 1] : roff[s + 1];
    std::vector<int> ix, iy, ty, rix, riy;
    std::vector<float> amp, sn, cs, sn2, cs2, sig;
    for (int s = 0; s < S; s++) {
        auto &a = c->acq[s];
        ix.insert(ix.end(), a.ix.begin(), a.ix.end());
        iy.insert(iy.end(), a.iy.begin(), a.iy.end());
        ty.insert(ty.end(), a.type.begin(), a.type.end());
        amp.insert(amp.end(), a.amp.begin(), a.amp.end());
        sn.insert(sn.end(), a.sn.begin(), a.sn.end());
        cs.insert(cs.end(), a.cs.begin(), a.cs.end());
        sn2.insert(sn2.end(), a.sn2.begin(), a.sn2.end());
        cs2.insert(cs2.end(), a.cs2.begin(), a.cs2.end());
        sig.insert(sig.end(), a.sig.begin(), a.sig.end());
        rix.insert(rix.end(), a.rix.begin(), a.rix.end());
        riy.insert(riy.end(), a.riy.begin(), a.riy.end());
        for (int t : a.type)
            if (t >= 2 && t <= 4)
                c->has_force = true;
    }
    // one allocation: ints then floats, 256-byte aligned pieces
    auto al = [](size_t n) { return (n + 63) / 64 * 64; };
    size_t ni = al(S + 1) * 2 + al(S) + al(ns_src) * 3 + al(nrec) * 2 + al(coloff.size()) + al(colidx.size());
    size_t nf = al(ns_src) * 5 + al((size_t)ns_src * NT);
    std::vector<int> hi(ni, 0);
    std::vector<float> hf(nf, 0.f);
    size_t pi = 0, pf = 0;
    auto puti = [&](const std::vector<int> &v, size_t n) { std::copy(v.begin(), v.end(), hi.begin() + pi); size_t o = pi; pi += al(n); return o; };
    auto putf = [&](const std::vector<float> &v, size_t n) { std::copy(v.begin(), v.end(), hf.begin() + pf); size_t o = pf; pf += al(n); return o; };
    size_t o_soff = puti(soff, S + 1), o_roff = puti(roff, S + 1), o_last = puti(last, S);
    size_t o_ix = puti(ix, ns_src), o_iy = puti(iy, ns_src), o_ty = puti(ty, ns_src);
    size_t o_rix = puti(rix, nrec), o_riy = puti(riy, nrec);
    size_t o_coff = puti(coloff, coloff.size()), o_cidx = puti(colidx, colidx.size());
    size_t o_amp = putf(amp, ns_src), o_sn = putf(sn, ns_src), o_cs = putf(cs, ns_src), o_sn2 = putf(sn2, ns_src),
           o_cs2 = putf(cs2, ns_src), o_sig = putf(sig, (size_t)ns_src * NT);
    if (c->acq_buf) {
        CK(cudaFreeAsync(c->acq_buf, c->stream));
        for (auto &p : c->allocs)
            if (p == c->acq_buf)
                p = nullptr;
        c->acq_buf = nullptr;
    }
    if (c->d_sec) {
        CK(cudaFreeAsync(c->d_sec, c->stream));
        for (auto &p : c->allocs)
            if (p == c->d_sec)
                p = nullptr;
        c->d_sec = nullptr;
    }
    void *buf;
    int rc = dalloc(c, &buf, ni * sizeof(int) + nf * sizeof(float));
    if (rc)
        return rc;
    c->acq_buf = buf;
    CK(cudaMemcpyAsync(buf, hi.data(), ni * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    float *fb = reinterpret_cast<float *>(reinterpret_cast<char *>(buf) + ni * sizeof(int));
    CK(cudaMemcpyAsync(fb, hf.data(), nf * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
    int *ib = reinterpret_cast<int *>(buf);
    Acq &A = c->A;
    A.src_off = ib + o_soff, A.rec_off = ib + o_roff, A.last_type = ib + o_last;
    A.src_ix = ib + o_ix, A.src_iy = ib + o_iy, A.src_type = ib + o_ty;
    A.rec_ix = ib + o_rix, A.rec_iy = ib + o_riy;
    A.rec_col_off = ib + o_coff, A.rec_col_idx = ib + o_cidx;
    A.src_amp = fb + o_amp, A.src_sin = fb + o_sn, A.src_cos = fb + o_cs, A.src_sin2 = fb + o_sn2,
    A.src_cos2 = fb + o_cs2, A.signals = fb + o_sig;
    A.nt = NT;
    A.ns = c->cfg.ndt > 0 ? NT / c->cfg.ndt : 0;
    float *sec;
    rc = dalloc(c, (void **)&sec, sizeof(float) * (size_t)(nrec > 0 ? nrec : 1) * 5 * (A.ns > 0 ? A.ns : 1));
    if (rc)
        return rc;
    c->d_sec = sec;
    A.sec = sec;
    A.status = c->d_status;
    c->total_src = ns_src;
    c->total_rec = nrec;
    // the per-cell flags of the stress kernel that does the post work, where
    // the configuration lets it (its memory: one byte per cell and shot)
    if (c->d_cellflag) {
        CK(cudaFreeAsync(c->d_cellflag, c->stream));
        for (auto &p : c->allocs)
            if (p == c->d_cellflag)
                p = nullptr;
        c->d_cellflag = nullptr;
    }
    A.cell_flag = nullptr;
    if (c->postf && post_flags_apply(c->cfg)) {
        const size_t n = (size_t)S * c->cfg.ny * c->cfg.nx;
        std::vector<unsigned char> fl(n, 0);
        for (int s = 0; s < S; s++) {
            const auto &a = c->acq[s];
            unsigned char *f = fl.data() + (size_t)s * c->cfg.ny * c->cfg.nx;
            if (last[s] == 1)
                for (size_t k = 0; k < a.ix.size(); k++)
                    f[(size_t)(a.iy[k] - 1) * c->cfg.nx + (a.ix[k] - 1)] |= 1;
            for (size_t k = 0; k < a.rix.size(); k++)
                f[(size_t)(a.riy[k] - 1) * c->cfg.nx + (a.rix[k] - 1)] |= 2;
        }
        if ((rc = dalloc(c, (void **)&c->d_cellflag, n)))
            return rc;
        CK(cudaMemcpyAsync(c->d_cellflag, fl.data(), n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        A.cell_flag = c->d_cellflag;
    }
    c->acq_dirty = false;
    c->graph_dirty = true;
    return 0;
}

dim3 grid2d(const sofi_ctx *c)
{
    unsigned tx = (c->cfg.nx + BX - 1) / BX, ty = (c->cfg.ny + BY - 1) / BY;
    if (c->G.shot_fast)
        return dim3(tx * c->cfg.nshots, ty, 1);
    return dim3(tx, ty, c->cfg.nshots);
}

// The ISO / VTI stress kernel with sw cells per thread in x (0: one).
void launch_cell_s(const Geo &G, const Wave &W, const Model &M, int nd, int kind, bool visco, int sw, bool narrow,
                   int nx, int ny, int nshots, cudaStream_t st, const Acq *post = nullptr)
{
    narrow = narrow && sw == 4 && kind != AC && narrow_s_applies(visco, visco ? G.L : 0, W.fa_x != nullptr);
    const int cx = sw ? sw : 1, bxt = narrow ? 8 : BX, byt = BX * BY / bxt;
    const unsigned tx = (nx + cx * bxt - 1) / (cx * bxt), ty = (ny + byt - 1) / byt;
    const dim3 grd = G.shot_fast ? dim3(tx * nshots, ty, 1) : dim3(tx, ty, nshots);
    if (kind == AC)
        launch_stress_ac(G, W, M, nd, sw, grd, st);
    else if (kind == ISO)
        visco ? launch_stress_kv<ISO, true>(G, W, M, nd, sw, narrow, grd, st, post)
              : launch_stress_kv<ISO, false>(G, W, M, nd, sw, narrow, grd, st, post);
    else
        visco ? launch_stress_kv<VTI, true>(G, W, M, nd, sw, narrow, grd, st, post)
              : launch_stress_kv<VTI, false>(G, W, M, nd, sw, narrow, grd, st, post);
}

// The wave fields a step's kernels get: the gradient quantities of an FWI
// pass (Wave::fa_*) only on its forward steps, so that the backward steps and
// every run outside a pass use the kernels that do not write them; the store
// (Wave::fstore) only on the stored steps of a VELOCITY = 1 pass. All forward
// steps, stored or not, run the same kernels: a segment recomputed from a
// checkpoint then repeats the first run's arithmetic.
Wave step_wave(const sofi_ctx *c)
{
    Wave W = c->W;
    W.fstore = nullptr, W.fbase = c->F.base;
    if (!c->fwi || c->fwi_back)
        W.fa_x = W.fa_y = nullptr;
    else if (c->fwi_store_on && c->F.velocity)
        W.fstore = c->F.store;
    return W;
}

// One time step. `capture`: being recorded into the step graph, so no host-
// side step number exists (no timing events, no snapshot).
// The velocity kernel in the context's variant: c->vw cells per thread in x
// (2 or 4), else c->vrows rows per thread.
void launch_v(sofi_ctx *c, const Geo &G, cudaStream_t st)
{
    const sofi_config &cf = c->cfg;
    const int S = cf.nshots;
    const bool ac = cf.weq == SOFI_AC_ISO;  // acoustic: one cell per thread when not vectorised
    const int vw = c->vw;
    const Wave W = step_wave(c);
    const bool narrow = c->vnarrow && vw == 4 && narrow_v_applies(ac, W.fa_x != nullptr);
    const int R = (vw || ac) ? 1 : c->vrows, cx = vw ? vw : 1, bxt = narrow ? 8 : BX, byt = BX * BY / bxt;
    const unsigned tx = (cf.nx + cx * bxt - 1) / (cx * bxt), ty = (cf.ny + byt * R - 1) / (byt * R);
    const dim3 gv = G.shot_fast ? dim3(tx * S, ty, 1) : dim3(tx, ty, S);
    launch_velocity(G, W, c->M, c->nd, vw, R, narrow, ac, gv, st, c->fwi_back && !c->tuning ? &c->F : nullptr);
}

// 4th-order time stepping has no autotuning: four cells per thread in both
// updates unless SOFI_VROWS=1|2|4 (velocity) or SOFI_SW=0 (stress) asks for one.
static bool ab4_wide_s(const sofi_ctx *c)
{
    return !(c->sw_fixed && c->sw == 0);
}

// Autotuner of the velocity and (ISO / VTI) stress kernels. Which variant is
// fastest depends on the grid: several cells per thread issue the fewest
// loads but leave few blocks on a small grid. The candidates are timed (CUDA
// events, back-to-back launches) on the context's own arrays while a reset
// leaves them all zero -- every candidate maps that state to itself, so
// tuning changes nothing -- and the winners are cached per configuration for
// the process. SOFI_VROWS / SOFI_SW fix a choice.
struct Tuned {
    int vw, vrows, sw;
    bool vnarrow, snarrow;
};
std::mutex g_tune_mu;
std::map<std::string, Tuned> g_tune;

template <typename F>
int time_launches(sofi_ctx *c, F launch, float *ms)
{
    constexpr int kWarm = 2, kTimed = 8;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    for (int k = 0; k < kWarm; k++)
        launch();
    cudaEventRecord(e0, c->stream);
    for (int k = 0; k < kTimed; k++)
        launch();
    cudaEventRecord(e1, c->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess)
        e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess)
        return fail(SOFI_E_CUDA, "autotune timing: %s", cudaGetErrorString(e));
    CK(cudaGetLastError());
    return 0;
}

// The narrow blocks are worth timing where the wide four-cell tiles (128
// columns) leave at least 8 % of a row's last blocks idle (nx = 400: 22 %).
static bool narrow_useful(int nx)
{
    const int w = (nx + 4 * BX - 1) / (4 * BX) * (4 * BX);
    return (w - nx) * 100 >= 8 * w;
}

static bool post_fused(const sofi_ctx *c);

static int autotune_(sofi_ctx *c);

// The tuner's launches run the plain kernels: none of them is a step (no step
// counter), and on a backward FWI step they carry no adjoint injection or
// density term.
int autotune(sofi_ctx *c)
{
    c->tuning = true;
    const int rc = autotune_(c);
    c->tuning = false;
    return rc;
}

static int autotune_(sofi_ctx *c)
{
    c->tuned = true;
    if (c->G.ab4)
        return 0;
    const sofi_config &cf = c->cfg;
    const int kind = kind_of(cf.weq);
    const bool visco = is_visco(cf.weq);
    const bool tune_s = kind != TTI && !c->sw_fixed;
    if (c->tune_fixed && !tune_s)
        return 0;
    char key[200];
    snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d", c->device, c->nd, cf.nx, cf.ny, cf.nshots,
             c->G.shot_fast, c->G.abs_type, cf.fw, cf.free_surf, cf.boundary, kind, visco ? c->G.L : -1,
             c->nmodels);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            if (!c->tune_fixed)
                c->vw = it->second.vw, c->vrows = it->second.vrows, c->vnarrow = it->second.vnarrow;
            if (tune_s)
                c->sw = it->second.sw, c->snarrow = it->second.snarrow;
            c->graph_dirty = true;
            return 0;
        }
    }
    if (!c->pristine)
        return 0;  // state not known to be zero: keep the default variants
    Geo G = c->G;
    G.step_ctr = nullptr;  // tuning launches are not steps
    Tuned pick{c->vw, c->vrows, c->sw, c->vnarrow, c->snarrow};
    float best = 1e30f, ms = 0.f;
    int rc;
    // two interleaved rounds over the candidates, each candidate's best time:
    // the first launches of a run can meet clocks still ramping up or a cold
    // L2, which would otherwise penalise whichever candidate goes first
    constexpr int kRounds = 2;
    if (!c->tune_fixed) {
        // {cells per thread, rows per thread, narrow blocks}; the acoustic update
        // has no narrow form.
        const bool ac = cf.weq == SOFI_AC_ISO;
        const int all[4][3] = {{4, 1, 0}, {2, 1, 0}, {0, 1, 0}, {4, 1, 1}};
        int cand[4][3], nc = 0;
        for (auto &cd : all)
            if (!(cd[2] && (ac || !narrow_useful(cf.nx))))
                std::copy(cd, cd + 3, cand[nc++]);
        float t[4] = {1e30f, 1e30f, 1e30f, 1e30f};
        for (int r = 0; r < kRounds; r++)
            for (int k = 0; k < nc; k++) {
                c->vw = cand[k][0], c->vrows = cand[k][1], c->vnarrow = cand[k][2];
                if ((rc = time_launches(c, [&] { launch_v(c, G, c->stream); }, &ms)))
                    return rc;
                t[k] = ms < t[k] ? ms : t[k];
            }
        for (int k = 0; k < nc; k++)
            if (t[k] < best)
                best = t[k], pick.vw = cand[k][0], pick.vrows = cand[k][1], pick.vnarrow = cand[k][2];
        c->vw = pick.vw, c->vrows = pick.vrows, c->vnarrow = pick.vnarrow;
    }
    if (tune_s) {
        // {cells per thread, narrow blocks}
        const int cand[4][2] = {{4, 0}, {2, 0}, {0, 0}, {4, 1}};
        const int nc = (kind != AC && narrow_useful(cf.nx) && narrow_s_applies(visco, visco ? c->G.L : 0, false)) ? 4 : 3;
        float t[4] = {1e30f, 1e30f, 1e30f, 1e30f};
        for (int r = 0; r < kRounds; r++)
            for (int k = 0; k < nc; k++) {
                const int w = cand[k][0];
                const bool nw = cand[k][1] != 0;
                if ((rc = time_launches(c,
                                        [&] {
                                            launch_cell_s(G, step_wave(c), c->M, c->nd, kind, visco, w, nw, cf.nx,
                                                          cf.ny, cf.nshots, c->stream);
                                        },
                                        &ms)))
                    return rc;
                t[k] = ms < t[k] ? ms : t[k];
            }
        // where the one-cell kernel would do the post work (post_fused), it
        // saves a k_post launch per step: on launch-bound grids (at most
        // 512 x 512 cells) credit it with one, timed on an empty acquisition
        // and a zero step count (it then reads only the zero state and
        // writes nothing); one shot, as d_noacq holds two ints
        const int keep_sw = c->sw;
        c->sw = 0;
        const bool fusable = cf.nshots == 1 && (long long)cf.nx * cf.ny <= 512 * 512 &&
                             (kind == ISO || kind == VTI) && post_fused(c);
        c->sw = keep_sw;
        if (fusable && !c->d_noacq && (rc = dalloc(c, (void **)&c->d_noacq, 2 * sizeof(int))))
            return rc;
        if (fusable) {
            Geo Gp = G;
            Gp.step_ctr = c->d_noacq;
            Acq E = c->A;
            E.src_off = c->d_noacq, E.last_type = c->d_noacq, E.rec_col_off = nullptr;
            const dim3 pg((cf.nx + 127) / 128, 1);
            float tp = 1e30f;
            for (int r = 0; r < kRounds; r++) {
                if ((rc = time_launches(c,
                                        [&] {
                                            if (visco)
                                                DISPATCH_ND(c->nd, (launch_pdl(k_post<ND, true, false>, pg, 128, 0,
                                                                               c->stream, Gp, step_wave(c), c->M, E)))
                                            else
                                                DISPATCH_ND(c->nd, (launch_pdl(k_post<ND, false, false>, pg, 128, 0,
                                                                               c->stream, Gp, step_wave(c), c->M, E)))
                                        },
                                        &ms)))
                    return rc;
                tp = ms < tp ? ms : tp;
            }
            t[2] -= tp;  // cand[2]: one cell per thread
        }
        best = 1e30f;
        for (int k = 0; k < nc; k++)
            if (t[k] < best)
                best = t[k], pick.sw = cand[k][0], pick.snarrow = cand[k][1] != 0;
        c->sw = pick.sw, c->snarrow = pick.snarrow;
    }
    c->graph_dirty = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = Tuned{c->vw, c->vrows, c->sw, c->vnarrow, c->snarrow};
    return 0;
}

// Whether the one-cell ISO / VTI stress kernel does k_post's work in this
// step (k_update_s_post, and k_update_s_post_fwi on the steps of an FWI
// pass): no free surface (its correction needs the column's updated rows), no
// moment-tensor source (it reaches a neighbouring cell), few sources per shot
// (a flagged cell scans them), 2nd-order time.
constexpr size_t kFusedSources = 8;
static bool post_fused(const sofi_ctx *c)
{
    const int kind = kind_of(c->cfg.weq);
    if (!c->postf || !c->A.cell_flag || c->sw != 0 || (kind != ISO && kind != VTI) || c->cfg.free_surf ||
        c->G.ab4)
        return false;
    for (const auto &a : c->acq)
        if ((!a.type.empty() && a.type.back() == 5) || a.ix.size() > kFusedSources)
            return false;
    return true;
}

int launch_step(sofi_ctx *c, int nt, bool capture = false)
{
    const sofi_config &cf = c->cfg;
    cudaStream_t st = c->stream;
    Geo &G = c->G;
    dim3 grd = grid2d(c);
    int S = cf.nshots;
    int nb = (S + 127) / 128;
    int kind = kind_of(cf.weq);
    bool visco = is_visco(cf.weq);
    const bool fused_post = post_fused(c);
    // a backward FWI step without a free surface: the stress kernel also
    // correlates (the post kernel then changes no stress)
    const bool conv_fused = c->fwi_back && !cf.free_surf && kind == ISO && !visco && !G.ab4;
    if (c->has_force) {
        launch_pdl(k_force_src, nb, 128, 0, st, G, c->W, c->M, c->A);
        c->launches++;
    }
    if (G.ab4) {  // 4th order: every block of the velocity kernel reads the step number
        launch_ab4_begin(G, st);
        c->launches++;
    }
    bool timed = !capture && c->time_every > 0 && (nt % c->time_every) == 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (timed) {
        if (c->tev_used + 3 > c->tev.size()) {
            for (int k = 0; k < 3; k++) {
                cudaEvent_t e;
                CK(cudaEventCreate(&e));
                c->tev.push_back(e);
            }
        }
        e0 = c->tev[c->tev_used], e1 = c->tev[c->tev_used + 1], e2 = c->tev[c->tev_used + 2];
        c->tev_used += 3;
        CK(cudaEventRecord(e0, st));
    }
    if (G.ab4)
        launch_ab4_v(G, c->W, c->M, c->nd, c->vw != 0, grd, st);
    else
        launch_v(c, G, st);
    c->launches++;
    if (timed)
        CK(cudaEventRecord(e1, st));
    if (cf.boundary) {
        k_wrap_x<<<dim3((cf.ny + 127) / 128, S), 128, 0, st>>>(G, c->W.vx, c->W.vy, nullptr, c->nd);
        c->launches++;
    }
    if (timed && cf.boundary)
        CK(cudaEventRecord(e1, st));
    if (G.ab4) {
        launch_ab4_s(G, c->W, c->M, c->nd, visco, ab4_wide_s(c), grd, st);
    } else if (kind == TTI && c->tti_split) {
        c->launches++;
        launch_tti_split(G, c->W, c->M, c->nd, visco, grd, st);
    } else if (kind == TTI && c->tti_fused) {
        launch_tti_fused(G, c->W, c->M, c->nd, visco, G.abs_type == 1, grd, st);
    } else if (kind == TTI) {
        launch_tti_tiles(G, c->W, c->M, c->nd, visco, G.abs_type == 1, st);
    } else if (conv_fused) {
        const int cx = c->sw ? c->sw : 1;
        const dim3 sg((cf.nx + cx * BX - 1) / (cx * BX), (cf.ny + BY - 1) / BY, 1);
        launch_stress_bwd(G, step_wave(c), c->M, c->F, c->nd, c->sw, sg, st, fused_post ? &c->A : nullptr);
    } else {
        launch_cell_s(G, step_wave(c), c->M, c->nd, kind, visco, c->sw, c->snarrow, cf.nx, cf.ny, S, st,
                      fused_post ? &c->A : nullptr);
    }
    c->launches++;
    if (timed)
        CK(cudaEventRecord(e2, st));
    dim3 pg((cf.nx + 127) / 128, S);
    if (fused_post) {
    } else if (kind == TTI) {
        DISPATCH_ND(c->nd, (launch_pdl(k_post<ND, false, true>, pg, 128, 0, st, G, c->W, c->M, c->A)))
    } else if (visco) {
        DISPATCH_ND(c->nd, (launch_pdl(k_post<ND, true, false>, pg, 128, 0, st, G, c->W, c->M, c->A)))
    } else {
        DISPATCH_ND(c->nd, (launch_pdl(k_post<ND, false, false>, pg, 128, 0, st, G, c->W, c->M, c->A)))
    }
    c->launches += fused_post ? 0 : 1;
    if (cf.boundary) {
        k_wrap_x<<<dim3((cf.ny + 127) / 128, S), 128, 0, st>>>(G, c->W.sxx, c->W.syy, c->W.sxy, c->nd);
        c->launches++;
    }
    if (c->fwi && (c->fwi_back || c->fwi_store_on)) {  // time_loop.c:288-296
        if (c->fwi_back) {
            if (!conv_fused) {  // else the stress kernel has correlated
                launch_fwi_conv(G, c->W, c->M, c->F, st);
                c->launches++;
            }
        } else if (!c->F.velocity) {  // VELOCITY = 1: the stress kernel stored the step
            launch_fwi_store(G, c->W, c->F, st);
            c->launches++;
        }
    }
    if (!capture && !c->fwi_nosnap && cf.snap && nt >= cf.snap_first && nt <= cf.snap_last &&
        (nt == cf.snap_first || (cf.snap_inc > 0 && (nt - cf.snap_first) % cf.snap_inc == 0)) &&
        c->nsnap < c->snap_total) {
        long long n = (long long)c->snap_nx * c->snap_ny;
        long long frame_stride = n * 5 * c->snap_total;
        float *out = c->d_snap + (long long)c->nsnap * 5 * n;
        dim3 sg((unsigned)((n + 127) / 128), S);
        DISPATCH_ND(c->nd, (k_snap<ND><<<sg, 128, 0, st>>>(G, c->W, c->M, out, c->snap_nx, c->snap_ny, cf.idx,
                                                          cf.idy, cf.snap, frame_stride)));
        c->nsnap++;
        c->launches++;
    }
    return 0;
}

int check_status(sofi_ctx *c)
{
    std::vector<int> st(c->cfg.nshots);
    CK(cudaMemcpyAsync(st.data(), c->d_status, sizeof(int) * st.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int s = 0; s < c->cfg.nshots; s++)
        if (st[s])
            return fail(SOFI_E_UNSTABLE, "shot %d: simulation is unstable (NaN at the probe cell after step %d)", s,
                        st[s]);
    return 0;
}

int copy_2d_in(sofi_ctx *c, float *dst, const float *host, long rs, long cs)
{
    const sofi_config &cf = c->cfg;
    float *d0 = dst + (long long)HY * c->G.pitch + HX;
    if (cs == 1) {
        CK(cudaMemcpy2DAsync(d0, sizeof(float) * c->G.pitch, host, sizeof(float) * rs, sizeof(float) * cf.nx, cf.ny,
                             cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return 0;
    }
    std::vector<float> tmp((size_t)cf.nx * cf.ny);
    for (int j = 0; j < cf.ny; j++)
        for (int i = 0; i < cf.nx; i++)
            tmp[(size_t)j * cf.nx + i] = host[(long long)j * rs + (long long)i * cs];
    CK(cudaMemcpy2DAsync(d0, sizeof(float) * c->G.pitch, tmp.data(), sizeof(float) * cf.nx, sizeof(float) * cf.nx,
                         cf.ny, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

float *field_ptr(sofi_ctx *c, int shot, const char *name)
{
    long long so = (long long)shot * c->G.fsz;
    if (!strcmp(name, "vx")) return c->W.vx + so;
    if (!strcmp(name, "vy")) return c->W.vy + so;
    if (!strcmp(name, "sxx")) return c->W.sxx + so;
    if (!strcmp(name, "syy")) return c->W.syy + so;
    if (!strcmp(name, "sxy")) return c->W.sxy + so;
    size_t n = strlen(name);
    if ((name[0] == 'r' || name[0] == 'p' || name[0] == 'q') && n == 2 && name[1] >= '1' && name[1] <= '8') {
        int l = name[1] - '1';
        if (l >= c->G.L)
            return nullptr;
        float *b = name[0] == 'r' ? c->W.r : (name[0] == 'p' ? c->W.p : c->W.q);
        if (c->G.ab4)  // the level the last step wrote
            b += (long long)(c->step & 3) * c->W.ab_mlvl;
        return b + ((long long)shot * c->G.L + l) * c->G.fsz;
    }
    return nullptr;
}

}  // namespace

extern "C" {

const char *sofi_last_error(void) { return g_err.c_str(); }
int sofi_abi_version(void) { return SOFI_ABI_VERSION; }

int sofi_device_bytes(const sofi_config *cfg, long long *bytes)
{
    int rc = check_config(cfg);
    if (rc)
        return rc;
    *bytes = fields_bytes(*cfg);
    return 0;
}

int sofi_stream_priority_range(int device, int *least, int *greatest)
{
    if (!least || !greatest)
        return fail(SOFI_E_ARG, "null argument");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(SOFI_E_NODEV, "no CUDA device available: %s", cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return fail(SOFI_E_ARG, "device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));
    CK(cudaDeviceGetStreamPriorityRange(least, greatest));
    return 0;
}

int sofi_device_memory(int device, long long *free_bytes, long long *total_bytes)
{
    if (!free_bytes || !total_bytes)
        return fail(SOFI_E_ARG, "null argument");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(SOFI_E_NODEV, "no CUDA device available: %s", cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return fail(SOFI_E_ARG, "device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));
    size_t f = 0, t = 0;
    CK(cudaMemGetInfo(&f, &t));
    *free_bytes = (long long)f, *total_bytes = (long long)t;
    return 0;
}

int sofi_create(const sofi_config *cfg, int device, sofi_ctx **out)
{
    return sofi_create_with_priority(cfg, device, 0, out);
}

int sofi_create_with_priority(const sofi_config *cfg, int device, int priority, sofi_ctx **out)
{
    if (!out)
        return fail(SOFI_E_ARG, "null output pointer");
    *out = nullptr;
    int rc = check_config(cfg);
    if (rc)
        return rc;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(SOFI_E_NODEV, "no CUDA device available: %s", cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return fail(SOFI_E_ARG, "device %d out of range (%d devices)", device, ndev);
    CK(cudaSetDevice(device));
    {
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        priority = priority < greatest ? greatest : (priority > least ? least : priority);
    }
    sofi_ctx *c = new sofi_ctx();
    c->cfg = *cfg;
    c->device = device;
    c->nd = cfg->fdorder / 2;
    c->nmodels = cfg->shared_model ? 1 : cfg->nshots;
    c->acq.resize(cfg->nshots);
    if (const char *e = getenv("SOFI_VROWS"))
    {
        // SOFI_VROWS: "w4" / "w2" cells per thread in x, "n4" four cells on
        // narrow blocks, "1" / "2" / "4" rows per thread
        const bool wide = e[0] == 'w' || e[0] == 'n';
        const int v = wide ? atoi(e + 1) : atoi(e);
        c->vw = wide ? (v == 2 && e[0] == 'w' ? 2 : 4) : 0;
        c->vnarrow = e[0] == 'n';
        c->vrows = (v == 2 || v == 4) ? v : 1;
        c->tune_fixed = true;
    }
    if (const char *e = getenv("SOFI_SW")) {  // "4" / "2" / "0" cells per thread, "n4" four on narrow blocks
        const int v = e[0] == 'n' ? 4 : atoi(e);
        c->sw = (v == 2 || v == 4) ? v : 0;
        c->snarrow = e[0] == 'n';
        c->sw_fixed = true;
    }
    if (const char *e = getenv("SOFI_POSTF"))
        c->postf = atoi(e) != 0;
    if (const char *e = getenv("SOFI_TTI")) {  // "split", "fused"; else the tiled one-pass form
        c->tti_split = strcmp(e, "split") == 0;
        c->tti_fused = strcmp(e, "fused") == 0;
    }
    e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, priority);
    if (e != cudaSuccess) {
        delete c;
        return fail(SOFI_E_CUDA, "stream creation: %s", cudaGetErrorString(e));
    }
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    Geo &G = c->G;
    G.nx = cfg->nx, G.ny = cfg->ny, G.pitch = pitch_for(cfg->nx), G.nshots = cfg->nshots;
    G.fsz = (long long)G.pitch * (cfg->ny + 2 * HY);
    G.fw = cfg->fw, G.fw2 = 2 * cfg->fw;
    G.abs_type = cfg->fw > 0 ? cfg->abs_type : 0;
    G.free_surf = cfg->free_surf, G.boundary = cfg->boundary;
    G.L = is_visco(cfg->weq) ? cfg->L : 0;
    G.model_stride_on = cfg->shared_model ? 0 : 1;
    G.el_tti_rb_short = (cfg->weq == SOFI_EL_TTI);
    G.shot_fast = (cfg->shared_model && cfg->nshots > 1) ? 1 : 0;
    G.seismo = cfg->seismo, G.ndt = cfg->ndt;
    G.ab4 = cfg->fdorder_time == 4;
    G.dhi4 = (float)(1.0 / (double)cfg->dh);
    c->W.ab_lvl = (long long)G.fsz * cfg->nshots;
    if (const char *e = getenv("SOFI_SHOT_ORDER"))
        G.shot_fast = G.shot_fast && strcmp(e, "slow") != 0;
    // subgrid_bounds.c:65-66,260-270 (one rank); without a frame the whole grid is interior
    int fw = G.abs_type ? cfg->fw : 0;
    G.gx2 = fw, G.gx3 = cfg->nx - fw, G.gy2 = fw, G.gy3 = cfg->ny - fw;
    if (cfg->free_surf)
        G.gy2 = 0;
    if (cfg->boundary)
        G.gx2 = 0, G.gx3 = cfg->nx;
    G.dt = cfg->dt, G.dh = cfg->dh;
    G.dtdh = cfg->dt / cfg->dh;
    G.dhi = 1.0f / cfg->dh;
    G.dthalbe = cfg->dt / 2.0f;
    for (int k = 0; k < 7; k++)
        G.hc[k] = (float)kHolberg[cfg->maxrelerror][c->nd - 1][k];
    // wavefields
    size_t f = (size_t)G.fsz * cfg->nshots * sizeof(float);
    float **w[5] = {&c->W.vx, &c->W.vy, &c->W.sxx, &c->W.syy, &c->W.sxy};
    for (auto p : w) {
        if (p == &c->W.syy && cfg->weq == SOFI_AC_ISO)
            continue;  // initmem_wavefield.c:34: one pressure array
        if ((rc = dalloc(c, (void **)p, f)))
            goto bad;
    }
    if (cfg->weq == SOFI_AC_ISO)
        c->W.syy = c->W.sxx;
    if (G.L) {
        float **m[3] = {&c->W.r, &c->W.p, &c->W.q};
        for (auto p : m)
            if ((rc = dalloc(c, (void **)p, f * G.L * (G.ab4 ? 4 : 1))))
                goto bad;
    }
    c->W.ab_mlvl = (long long)G.fsz * cfg->nshots * G.L;
    if (G.ab4) {
        float **h[6] = {&c->W.svx4, &c->W.svy4, &c->W.hxx4, &c->W.hyy4, &c->W.hxy4, &c->W.hyx4};
        for (auto p : h)
            if ((rc = dalloc(c, (void **)p, f * 4)))
                goto bad;
    }
    if (G.abs_type == 1) {
        size_t px = sizeof(float) * (size_t)cfg->nshots * cfg->ny * G.fw2;
        size_t py = sizeof(float) * (size_t)cfg->nshots * G.fw2 * cfg->nx;
        float **a[4] = {&c->W.psi_sxx_x, &c->W.psi_sxy_x, &c->W.psi_vxx, &c->W.psi_vyx};
        float **b[4] = {&c->W.psi_syy_y, &c->W.psi_sxy_y, &c->W.psi_vyy, &c->W.psi_vxy};
        // the fused TTI stress kernel keeps the derivative memory in two buffers
        const int nb = (kind_of(cfg->weq) == TTI && !c->tti_split) ? 2 : 1;
        G.psi_pp = nb == 2;
        G.psi_xsz = (long long)cfg->nshots * cfg->ny * G.fw2;
        G.psi_ysz = (long long)cfg->nshots * G.fw2 * cfg->nx;
        for (int k = 0; k < 4; k++)
            if ((rc = dalloc(c, (void **)a[k], px * (k >= 2 ? nb : 1))))
                goto bad;
        for (int k = 0; k < 4; k++)
            if ((rc = dalloc(c, (void **)b[k], py * (k >= 2 ? nb : 1))))
                goto bad;
        // profile vectors: 12 x 2FW, one block
        float *pv;
        if ((rc = dalloc(c, (void **)&pv, sizeof(float) * 12 * G.fw2)))
            goto bad;
        const float **slots[12] = {&c->M.K_x, &c->M.a_x, &c->M.b_x, &c->M.K_x_half, &c->M.a_x_half,
                                   &c->M.b_x_half, &c->M.K_y, &c->M.a_y, &c->M.b_y, &c->M.K_y_half,
                                   &c->M.a_y_half, &c->M.b_y_half};
        for (int k = 0; k < 12; k++)
            *slots[k] = pv + (size_t)k * G.fw2;
    }
    if (kind_of(cfg->weq) == TTI && c->tti_split) {
        if ((rc = dalloc(c, (void **)&c->W.draw, f * 4)) || (rc = dalloc(c, (void **)&c->W.dcor, f * 4)))
            goto bad;
    }
    for (const auto &n : needed_fields(*cfg)) {
        float *p;
        if ((rc = dalloc(c, (void **)&p, (size_t)G.fsz * c->nmodels * sizeof(float))))
            goto bad;
        *slot_ptr(c->M, n.c_str(), true) = p;
    }
    if ((rc = dalloc(c, (void **)&c->d_status, sizeof(int) * (cfg->nshots + 2))))
        goto bad;
    c->G.step_ctr = c->d_status + cfg->nshots;  // zeroed with the status words
    c->F.bstep = c->d_status + cfg->nshots + 1; // the same
    if (const char *e = getenv("SOFI_GRAPH"))
        c->use_graph = atoi(e) != 0;
    if (const char *e = getenv("SOFI_PDL"))
        c->pdl = atoi(e) != 0;
    c->A.status = c->d_status;
    c->snap_total = count_snapshots(*cfg);
    if (c->snap_total) {
        c->snap_nx = (cfg->nx - 1) / cfg->idx + 1;
        c->snap_ny = (cfg->ny - 1) / cfg->idy + 1;
        size_t n = (size_t)c->snap_nx * c->snap_ny * 5 * c->snap_total * cfg->nshots;
        if ((rc = dalloc(c, (void **)&c->d_snap, n * sizeof(float))))
            goto bad;
    }
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        rc = fail(SOFI_E_CUDA, "initialisation: %s", cudaGetErrorString(e));
        goto bad;
    }
    *out = c;
    return 0;
bad:
    sofi_destroy(c);
    return rc;
}

int sofi_destroy(sofi_ctx *c)
{
    if (!c)
        return 0;
    cudaSetDevice(c->device);
    if (c->stream) {
        for (void *p : c->allocs)
            if (p)
                cudaFreeAsync(p, c->stream);
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
    }
    for (auto e : c->tev)
        cudaEventDestroy(e);
    for (auto e : c->run_ev)
        cudaEventDestroy(e);
    for (auto e : c->ev_free)
        cudaEventDestroy(e);
    drop_graphs(c);
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    delete c;
    return 0;
}

int sofi_set_hc(sofi_ctx *c, const float *hc)
{
    if (!c || !hc)
        return fail(SOFI_E_ARG, "null argument");
    c->graph_dirty = true;
    for (int k = 0; k < 7; k++)
        c->G.hc[k] = hc[k];
    return 0;
}

int sofi_set_model_field(sofi_ctx *c, int model, const char *name, const float *host, long row_stride,
                         long col_stride)
{
    if (!c || !name || !host)
        return fail(SOFI_E_ARG, "null argument");
    if (model < 0 || model >= c->nmodels)
        return fail(SOFI_E_ARG, "model index %d out of range (%d models)", model, c->nmodels);
    CK(cudaSetDevice(c->device));
    const float **slot = slot_ptr(c->M, name, is_visco(c->cfg.weq));
    if (!slot)
        return fail(SOFI_E_ARG, "unknown model field '%s'", name);
    if (!*slot)
        return fail(SOFI_E_ARG, "model field '%s' is not used by this wave equation", name);
    float *dst = const_cast<float *>(*slot) + (long long)model * c->G.fsz;
    return copy_2d_in(c, dst, host, row_stride, col_stride);
}

int sofi_set_model_vector(sofi_ctx *c, const char *name, const float *host, int n)
{
    if (!c || !name || !host)
        return fail(SOFI_E_ARG, "null argument");
    c->graph_dirty = true;
    CK(cudaSetDevice(c->device));
    if (!strcmp(name, "bip") || !strcmp(name, "cip") || !strcmp(name, "peta")) {
        if (n != c->G.L)
            return fail(SOFI_E_ARG, "%s needs L=%d values", name, c->G.L);
        float *d = !strcmp(name, "bip") ? c->M.bip : (!strcmp(name, "cip") ? c->M.cip : c->M.peta);
        for (int l = 0; l < n; l++)
            d[l] = host[l];
        return 0;
    }
    const float **slots[12] = {&c->M.K_x, &c->M.a_x, &c->M.b_x, &c->M.K_x_half, &c->M.a_x_half, &c->M.b_x_half,
                               &c->M.K_y, &c->M.a_y, &c->M.b_y, &c->M.K_y_half, &c->M.a_y_half, &c->M.b_y_half};
    for (int k = 0; k < 12; k++)
        if (!strcmp(name, kVectors[k])) {
            if (c->G.abs_type != 1)
                return fail(SOFI_E_ARG, "CPML profile '%s' given without a CPML frame", name);
            if (n != c->G.fw2)
                return fail(SOFI_E_ARG, "%s needs 2*FW=%d values", name, c->G.fw2);
            CK(cudaMemcpyAsync(const_cast<float *>(*slots[k]), host, sizeof(float) * n, cudaMemcpyHostToDevice,
                               c->stream));
            CK(cudaStreamSynchronize(c->stream));
            return 0;
        }
    return fail(SOFI_E_ARG, "unknown model vector '%s'", name);
}

int sofi_set_sources(sofi_ctx *c, int shot, int nsrc, const float *srcpos, const float *signals)
{
    if (!c || shot < 0 || shot >= c->cfg.nshots || nsrc < 0 || (nsrc && (!srcpos || !signals)))
        return fail(SOFI_E_ARG, "invalid source arguments");
    ShotAcq &a = c->acq[shot];
    a.ix.assign(nsrc, 0), a.iy.assign(nsrc, 0), a.type.assign(nsrc, 0);
    a.amp.assign(nsrc, 0.f), a.sn.assign(nsrc, 0.f), a.cs.assign(nsrc, 0.f), a.sn2.assign(nsrc, 0.f),
        a.cs2.assign(nsrc, 0.f);
    a.sig.assign(signals, signals + (size_t)nsrc * c->cfg.nt);
    for (int k = 0; k < nsrc; k++) {
        int ix = (int)srcpos[0 * nsrc + k], iy = (int)srcpos[1 * nsrc + k], t = (int)srcpos[7 * nsrc + k];
        if (ix < 1 || ix > c->cfg.nx || iy < 1 || iy > c->cfg.ny)
            return fail(SOFI_E_ARG, "source %d at grid (%d,%d) outside 1..%d x 1..%d", k, ix, iy, c->cfg.nx,
                        c->cfg.ny);
        if (t < 1 || t > 5)
            return fail(SOFI_E_ARG, "source %d has unsupported type %d", k, t);
        if (t == 5 && (iy < 2 || ix < 2))
            return fail(SOFI_E_ARG, "moment-tensor source %d needs i, j >= 2", k);
        a.ix[k] = ix, a.iy[k] = iy, a.type[k] = t;
        a.amp[k] = srcpos[5 * nsrc + k];
        // update_v_interior.c:55 (azimuth, float radians) and eqsource.c:39 (dip)
        float azi_rad = (float)(srcpos[6 * nsrc + k] * M_PI / 180);
        a.sn[k] = (float)sin(azi_rad), a.cs[k] = (float)cos(azi_rad);
        float dip = (float)(srcpos[6 * nsrc + k] * M_PI / 180.0);
        a.sn2[k] = (float)sin(2 * dip), a.cs2[k] = (float)cos(2 * dip);
    }
    c->acq_dirty = true;
    return 0;
}

int sofi_set_receivers(sofi_ctx *c, int shot, int ntr, const int *ix, const int *iy)
{
    if (!c || shot < 0 || shot >= c->cfg.nshots || ntr < 0 || (ntr && (!ix || !iy)))
        return fail(SOFI_E_ARG, "invalid receiver arguments");
    for (int k = 0; k < ntr; k++)
        if (ix[k] < 1 || ix[k] > c->cfg.nx || iy[k] < 1 || iy[k] > c->cfg.ny)
            return fail(SOFI_E_ARG, "receiver %d at grid (%d,%d) outside the grid", k, ix[k], iy[k]);
    c->acq[shot].rix.assign(ix, ix + ntr);
    c->acq[shot].riy.assign(iy, iy + ntr);
    c->acq_dirty = true;
    return 0;
}

int sofi_reset(sofi_ctx *c, int shot)
{
    if (!c || shot < -1 || shot >= c->cfg.nshots)
        return fail(SOFI_E_ARG, "invalid shot");
    CK(cudaSetDevice(c->device));
    int s0 = shot < 0 ? 0 : shot, s1 = shot < 0 ? c->cfg.nshots : shot + 1;
    size_t f = (size_t)c->G.fsz * sizeof(float);
    for (int s = s0; s < s1; s++) {
        float *w[5] = {c->W.vx, c->W.vy, c->W.sxx, c->W.syy, c->W.sxy};
        for (auto p : w)
            CK(cudaMemsetAsync(p + (long long)s * c->G.fsz, 0, f, c->stream));
        if (c->G.L) {
            float *m[3] = {c->W.r, c->W.p, c->W.q};
            for (int k = 0; k < (c->G.ab4 ? 4 : 1); k++)
                for (auto p : m)
                    CK(cudaMemsetAsync(p + k * c->W.ab_mlvl + (long long)s * c->G.L * c->G.fsz, 0, f * c->G.L,
                                       c->stream));
        }
        if (c->G.ab4) {
            float *h[6] = {c->W.svx4, c->W.svy4, c->W.hxx4, c->W.hyy4, c->W.hxy4, c->W.hyx4};
            for (int k = 0; k < 4; k++)
                for (auto p : h)
                    CK(cudaMemsetAsync(p + k * c->W.ab_lvl + (long long)s * c->G.fsz, 0, f, c->stream));
        }
        if (c->G.abs_type == 1) {
            size_t px = sizeof(float) * (size_t)c->cfg.ny * c->G.fw2, py = sizeof(float) * (size_t)c->G.fw2 * c->cfg.nx;
            float *a[4] = {c->W.psi_sxx_x, c->W.psi_sxy_x, c->W.psi_vxx, c->W.psi_vyx};
            float *b[4] = {c->W.psi_syy_y, c->W.psi_sxy_y, c->W.psi_vyy, c->W.psi_vxy};
            for (int k = 0; k < 4; k++)
                for (int bb = 0; bb < ((k >= 2 && c->G.psi_pp) ? 2 : 1); bb++) {
                    CK(cudaMemsetAsync(a[k] + bb * c->G.psi_xsz + (long long)s * c->cfg.ny * c->G.fw2, 0, px,
                                       c->stream));
                    CK(cudaMemsetAsync(b[k] + bb * c->G.psi_ysz + (long long)s * c->G.fw2 * c->cfg.nx, 0, py,
                                       c->stream));
                }
        }
        if (c->W.draw) {
            CK(cudaMemsetAsync(c->W.draw + 4LL * s * c->G.fsz, 0, 4 * f, c->stream));
            CK(cudaMemsetAsync(c->W.dcor + 4LL * s * c->G.fsz, 0, 4 * f, c->stream));
        }
    }
    CK(cudaMemsetAsync(c->d_status, 0, sizeof(int) * (c->cfg.nshots + 2), c->stream));  // + step counters
    if (c->d_sec && !c->acq_dirty) {
        size_t n = (size_t)c->total_rec * 5 * (c->A.ns > 0 ? c->A.ns : 1);
        CK(cudaMemsetAsync(c->d_sec, 0, n * sizeof(float), c->stream));
    }
    c->step = 0;
    c->nsnap = 0;
    CK(cudaStreamSynchronize(c->stream));
    c->pristine = shot < 0;
    return 0;
}

// Whether steps first..first+n-1 need a direct launch (snapshot or timed step).
static bool chunk_has_event(const sofi_ctx *c, int first, int n)
{
    const sofi_config &cf = c->cfg;
    for (int nt = first; nt < first + n; nt++) {
        if (c->time_every > 0 && nt % c->time_every == 0)
            return true;
        if (cf.snap && nt >= cf.snap_first && nt <= cf.snap_last &&
            (nt == cf.snap_first || (cf.snap_inc > 0 && (nt - cf.snap_first) % cf.snap_inc == 0)))
            return true;
    }
    return false;
}

// Graph of kGraphSteps steps.
static int build_graph(sofi_ctx *c)
{
    cudaGraphExec_t &gx = c->graph_exec;
    if (gx) {
        cudaGraphExecDestroy(gx);
        gx = nullptr;
    }
    long long before = c->launches;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    for (int k = 0; k < kGraphSteps && !rc; k++)
        rc = launch_step(c, 0, true);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc)
        return rc;
    if (e != cudaSuccess)
        return fail(SOFI_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&gx, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return fail(SOFI_E_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
    c->graph_launches = c->launches - before;
    c->launches = before;
    c->graph_ok = true;
    return 0;
}

static int fwi_copy_state(sofi_ctx *c, float *buf, bool save);

int sofi_run(sofi_ctx *c, int nsteps)
{
    if (!c || nsteps < 0)
        return fail(SOFI_E_ARG, "invalid run arguments");
    if (c->step + nsteps > c->cfg.nt)
        return fail(SOFI_E_ARG, "step %d + %d exceeds NT=%d", c->step, nsteps, c->cfg.nt);
    CK(cudaSetDevice(c->device));
    pdl_flag() = c->pdl;  // every kernel of this run is launched from this thread
    if (c->G.abs_type == 1 && !c->M.K_x)
        return fail(SOFI_E_STATE, "CPML profiles not set");
    if (c->acq_dirty) {
        int rc = upload_acq(c);
        if (rc)
            return rc;
    }
    if (!c->tuned && c->step == 0 && nsteps > 0) {
        // an FWI pass's forward run tunes the plain kernels (step_wave drops
        // the gradient quantities while fwi_back is set), then runs the FWI
        // instantiations of the winners: 4, 2 or 1 cells per thread on wide blocks
        const bool fb = c->fwi_back;
        if (c->fwi)
            c->fwi_back = true;
        int rc = autotune(c);
        c->fwi_back = fb;
        if (rc)
            return rc;
        if (c->fwi && !c->fwi_back) {
            if (c->vw == 0)
                c->vrows = 1;
            c->vnarrow = c->snarrow = false;
            c->fwi_vw = c->vw, c->fwi_sw = c->sw;
            c->graph_dirty = true;
        }
    }
    c->pristine = false;
    CK(cudaEventRecord(c->ev0, c->stream));
    // the forward run of a checkpointed FWI pass keeps the state after steps K, 2K, ...
    const bool ckpt_fwd = c->fwi && c->fwi_K && !c->fwi_back && !c->fwi_store_on;
    int left = nsteps;
    while (left > 0) {
        const int lim = ckpt_fwd ? std::min(left, c->fwi_K - c->step % c->fwi_K) : left;
        if (c->use_graph && lim >= kGraphSteps && !chunk_has_event(c, c->step + 1, kGraphSteps)) {
            if (c->graph_dirty) {
                drop_graphs(c);
                c->graph_dirty = false;
            }
            if (!c->graph_ok) {
                int rc = build_graph(c);
                if (rc)
                    return rc;
            }
            CK(cudaGraphLaunch(c->graph_exec, c->stream));
            c->launches += c->graph_launches;
            c->step += kGraphSteps;
            left -= kGraphSteps;
        } else {
            int rc = launch_step(c, c->step + 1);
            if (rc)
                return rc;
            c->step++;
            left--;
        }
        if (ckpt_fwd && c->step % c->fwi_K == 0 && c->step < c->cfg.nt) {
            int rc = fwi_copy_state(c, c->fwi_ckpt + (size_t)(c->step / c->fwi_K - 1) * c->fwi_state, true);
            if (rc)
                return rc;
        }
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaGetLastError());
    c->run_pending = true;
    cudaEvent_t done;
    if (c->ev_free.empty()) {
        CK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    } else {
        done = c->ev_free.back();
        c->ev_free.pop_back();
    }
    c->run_ev.push_back(done);
    CK(cudaEventRecord(done, c->stream));
    return 0;
}

int sofi_pending_runs(sofi_ctx *c, int *pending)
{
    if (!c || !pending)
        return fail(SOFI_E_ARG, "null argument");
    CK(cudaSetDevice(c->device));
    while (!c->run_ev.empty()) {
        cudaError_t e = cudaEventQuery(c->run_ev.front());
        if (e == cudaErrorNotReady)
            break;
        if (e != cudaSuccess)
            return fail(SOFI_E_CUDA, "run completion: %s", cudaGetErrorString(e));
        c->ev_free.push_back(c->run_ev.front());
        c->run_ev.pop_front();
    }
    *pending = (int)c->run_ev.size();
    return 0;
}

int sofi_synchronize(sofi_ctx *c)
{
    if (!c)
        return fail(SOFI_E_ARG, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->run_pending) {
        CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
        c->run_pending = false;
    }
    for (size_t k = 0; k + 3 <= c->tev_used; k += 3) {
        float a = 0, b = 0;
        CK(cudaEventElapsedTime(&a, c->tev[k], c->tev[k + 1]));
        CK(cudaEventElapsedTime(&b, c->tev[k + 1], c->tev[k + 2]));
        c->t_v_ms += a, c->t_s_ms += b, c->t_count++;
    }
    c->tev_used = 0;
    return check_status(c);
}

int sofi_set_kernel_timing(sofi_ctx *c, int every)
{
    if (!c || every < 0)
        return fail(SOFI_E_ARG, "invalid timing arguments");
    CK(cudaStreamSynchronize(c->stream));
    c->time_every = every;
    c->tev_used = 0;
    c->t_v_ms = c->t_s_ms = 0;
    c->t_count = 0;
    return 0;
}

int sofi_kernel_time(sofi_ctx *c, const char *name, double *avg_ms, long long *count)
{
    if (!c || !name || !avg_ms || !count)
        return fail(SOFI_E_ARG, "null argument");
    int rc = sofi_synchronize(c);
    if (rc)
        return rc;
    double t;
    if (!strcmp(name, "update_v"))
        t = c->t_v_ms;
    else if (!strcmp(name, "update_s"))
        t = c->t_s_ms;
    else
        return fail(SOFI_E_ARG, "unknown timed kernel '%s'", name);
    *count = c->t_count;
    *avg_ms = c->t_count ? t / c->t_count : 0.0;
    return 0;
}

int sofi_get_stream(sofi_ctx *c, void **stream)
{
    if (!c || !stream)
        return fail(SOFI_E_ARG, "null argument");
    *stream = (void *)c->stream;
    return 0;
}

int sofi_velocity_variant(sofi_ctx *c, int *cells_per_thread, int *rows_per_thread)
{
    if (!c || !cells_per_thread || !rows_per_thread)
        return fail(SOFI_E_ARG, "null argument");
    const int vw = c->vw;
    *cells_per_thread = !vw ? 1 : c->G.ab4 ? 4 : vw;  // 4th order: four cells or one
    *rows_per_thread = (vw || c->G.ab4) ? 1 : c->vrows;
    return 0;
}

// The state a forward or backward FWI run carries from step to step: the
// wavefield (one shot, padded fields) and, with CPML, the eight memory arrays.
static std::vector<std::pair<float *, size_t>> fwi_state_parts(sofi_ctx *c)
{
    std::vector<std::pair<float *, size_t>> v;
    const size_t f = (size_t)c->G.fsz;
    for (float *p : {c->W.vx, c->W.vy, c->W.sxx, c->W.syy, c->W.sxy})
        v.push_back({p, f});
    if (c->G.abs_type == 1) {
        const size_t px = (size_t)c->cfg.ny * c->G.fw2, py = (size_t)c->G.fw2 * c->cfg.nx;
        for (float *p : {c->W.psi_sxx_x, c->W.psi_sxy_x, c->W.psi_vxx, c->W.psi_vyx})
            v.push_back({p, px});
        for (float *p : {c->W.psi_syy_y, c->W.psi_sxy_y, c->W.psi_vyy, c->W.psi_vxy})
            v.push_back({p, py});
    }
    return v;
}

// save: state -> buf; else buf -> state (buf null: zero the state)
static int fwi_copy_state(sofi_ctx *c, float *buf, bool save)
{
    size_t off = 0;
    for (auto &pt : fwi_state_parts(c)) {
        const size_t b = pt.second * sizeof(float);
        if (save)
            CK(cudaMemcpyAsync(buf + off, pt.first, b, cudaMemcpyDeviceToDevice, c->stream));
        else if (buf)
            CK(cudaMemcpyAsync(pt.first, buf + off, b, cudaMemcpyDeviceToDevice, c->stream));
        else
            CK(cudaMemsetAsync(pt.first, 0, b, c->stream));
        off += pt.second;
    }
    return 0;
}

static int fwi_set_step(sofi_ctx *c, int step, int base)
{
    c->step = step;
    CK(cudaMemcpyAsync(c->G.step_ctr, &step, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->F.bstep, &step, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_fwi_base, &base, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));  // the host ints above are locals
    return 0;
}

int sofi_fwi_begin(sofi_ctx *c, int velocity, int adjoint_type, const float *vp, const float *vs, const float *rho)
{
    if (!c || !vp || !vs || !rho)
        return fail(SOFI_E_ARG, "null argument");
    const sofi_config &cf = c->cfg;
    if (cf.weq != SOFI_EL_ISO || cf.nshots != 1 || c->G.ab4)
        return fail(SOFI_E_ARG, "FWI gradients need WEQ = EL_ISO, one shot, FDORDER_TIME = 2 and the plain kernels");
    if (cf.ndt != 1 || (cf.seismo != 1 && cf.seismo != 4))
        return fail(SOFI_E_ARG, "FWI gradients need NDT = 1 and vx / vy seismograms (SEISMO 1 or 4)");
    if ((velocity != 0 && velocity != 1) || adjoint_type < 1 || adjoint_type > 3)
        return fail(SOFI_E_ARG, "VELOCITY 0 / 1 and ADJOINT_TYPE 1-3 are supported");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    const size_t n = (size_t)cf.nx * cf.ny, f = (size_t)c->G.fsz * sizeof(float);
    int rc;
    // the whole forward run in the store when it fits, else checkpoints every K
    // steps (SOFI_FWI_CHECKPOINT=K forces it): memory (nseg - 1 + 1) states + K
    // slots, one extra forward run per pass whatever K is
    c->fwi_state = 0;
    for (auto &pt : fwi_state_parts(c))
        c->fwi_state += pt.second;
    const size_t slot = 5 * n * sizeof(float), state = c->fwi_state * sizeof(float);
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    const size_t reserve = (16 * n) * sizeof(float) + 2 * f + (64u << 20);
    const size_t have = (c->F.store ? c->fwi_slots * slot : 0) + (c->fwi_ckpt ? c->fwi_ckpt_cap * state : 0) + fr;
    int K = 0;
    if (const char *e = getenv("SOFI_FWI_CHECKPOINT"))
        K = atoi(e) > 0 ? (atoi(e) < cf.nt ? atoi(e) : cf.nt) : 0;
    if (!K && (size_t)cf.nt * slot + reserve > have) {
        K = (int)ceil(sqrt((double)cf.nt * (double)state / (double)slot));
        K = K < 1 ? 1 : (K > cf.nt ? cf.nt : K);
    }
    const int nseg = K ? (cf.nt + K - 1) / K : 1;
    const size_t slots = K ? (size_t)K : (size_t)cf.nt;
    const size_t nck = K ? (size_t)nseg : 0;  // nseg - 1 checkpoints + the backward state
    if (slots * slot + nck * state + reserve > have)
        return fail(SOFI_E_NOMEM, "the FWI pass needs %zu bytes of forward store and checkpoints, %zu free",
                    slots * slot + nck * state, have);
    if (slots > c->fwi_slots) {
        if ((rc = dalloc(c, (void **)&c->F.store, slots * slot)))
            return rc;
        c->fwi_slots = slots;
    }
    if (nck > c->fwi_ckpt_cap) {
        if ((rc = dalloc(c, (void **)&c->fwi_ckpt, nck * state)))
            return rc;
        c->fwi_ckpt_cap = nck;
    }
    c->fwi_tmp = nck ? c->fwi_ckpt + (nck - 1) * c->fwi_state : nullptr;
    c->fwi_K = K, c->fwi_nseg = nseg;
    c->fwi_store_on = K == 0;
    if (!c->F.px) {
        float **fl[] = {&c->F.px, &c->F.py, &c->F.g_lam, &c->F.g_mu, &c->F.g_rhos};
        for (int k = 0; k < 5; k++)
            if ((rc = dalloc(c, (void **)fl[k], n * sizeof(float))))
                return rc;
        float *m[3];
        for (int k = 0; k < 3; k++)
            if ((rc = dalloc(c, (void **)&m[k], n * sizeof(float))))
                return rc;
        c->F.vp = m[0], c->F.vs = m[1], c->F.rho = m[2];
        if ((rc = dalloc(c, (void **)&c->F.rc, 3 * n * sizeof(double))))
            return rc;
        float **wf[] = {&c->W.fa_x, &c->W.fa_y};
        for (auto p : wf)
            if ((rc = dalloc(c, (void **)p, f)))
                return rc;
        if ((rc = dalloc(c, (void **)&c->d_noacq, 2 * sizeof(int))) ||
            (rc = dalloc(c, (void **)&c->d_fwi_base, sizeof(int))))
            return rc;
        c->F.base = c->d_fwi_base;
    }
    CK(cudaMemsetAsync(c->d_fwi_base, 0, sizeof(int), c->stream));
    CK(cudaMemcpyAsync((void *)c->F.vp, vp, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync((void *)c->F.vs, vs, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync((void *)c->F.rho, rho, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    for (float *p : {c->F.g_lam, c->F.g_mu, c->F.g_rhos})
        CK(cudaMemsetAsync(p, 0, n * sizeof(float), c->stream));
    launch_fwi_coef((int)n, c->F, c->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    c->F.nt = cf.nt, c->F.velocity = velocity, c->F.adjoint = adjoint_type;
    // the forward steps run the kernels whose bodies write the gradient
    // quantities, in the variant the autotuner picks for plain steps of this
    // grid at the pass's first sofi_run (four cells per thread until then;
    // SOFI_VROWS / SOFI_SW keep the variant they fix)
    if (!c->tune_fixed)
        c->vw = 4, c->vrows = 1;
    if (!c->sw_fixed)
        c->sw = 4;
    c->tuned = false;
    c->vnarrow = c->snarrow = false;
    c->fwi_vw = c->vw, c->fwi_sw = c->sw;
    c->fwi = true, c->fwi_back = false, c->graph_dirty = true;
    return 0;
}

int sofi_fwi_backward(sofi_ctx *c, const float *adj_x, const float *adj_y)
{
    if (!c || !adj_x || !adj_y)
        return fail(SOFI_E_ARG, "null argument");
    if (!c->fwi || c->fwi_back)
        return fail(SOFI_E_STATE, "sofi_fwi_begin first");
    int rc = sofi_synchronize(c);
    if (rc)
        return rc;
    if (c->step != c->cfg.nt)
        return fail(SOFI_E_STATE, "the forward run has done %d of NT = %d steps", c->step, c->cfg.nt);
    // receivers grouped by cell, each cell's in the reference's order
    const ShotAcq &a = c->acq[0];
    const int ntr = (int)a.rix.size(), NT = c->cfg.nt;
    std::map<std::pair<int, int>, std::vector<int>> cells;
    std::vector<std::pair<int, int>> order;
    for (int l = 0; l < ntr; l++) {
        auto key = std::make_pair(a.riy[l], a.rix[l]);
        if (!cells.count(key))
            order.push_back(key);
        cells[key].push_back(l);
    }
    // the backward velocity kernel finds a cell's receivers through a map of
    // the grid (k + 1 at receiver cell k)
    const size_t n = (size_t)c->cfg.nx * c->cfg.ny;
    std::vector<int> off(1, 0), rec, map(n, 0);
    for (auto &k : order) {
        for (int l : cells[k])
            rec.push_back(l);
        off.push_back((int)rec.size());
        map[(size_t)(k.first - 1) * c->cfg.nx + (k.second - 1)] = (int)off.size() - 1;
    }
    const size_t nc = order.size();
    if (nc + 1 > c->fwi_cells_cap || !c->F.adj) {
        int *ib;
        float *adj;
        const size_t cap = (nc + 1) > 1 ? nc + 1 : 2;
        if ((rc = dalloc(c, (void **)&ib, (cap + (size_t)ntr) * sizeof(int))) ||
            (rc = dalloc(c, (void **)&adj, 2 * (size_t)(ntr > 0 ? ntr : 1) * NT * sizeof(float))))
            return rc;
        c->F.cell_off = ib, c->F.cell_rec = ib + cap;
        c->F.adj = adj;
        c->fwi_cells_cap = cap;
    }
    if (!c->F.cell_map) {
        int *mp;
        if ((rc = dalloc(c, (void **)&mp, n * sizeof(int))))
            return rc;
        c->F.cell_map = mp;
    }
    CK(cudaMemcpyAsync((void *)c->F.cell_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync((void *)c->F.cell_map, map.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    if (nc)
        CK(cudaMemcpyAsync((void *)c->F.cell_rec, rec.data(), rec.size() * sizeof(int), cudaMemcpyHostToDevice,
                           c->stream));
    const size_t m = (size_t)ntr * NT;
    CK(cudaMemcpyAsync((void *)c->F.adj, adj_x, m * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync((void *)(c->F.adj + m), adj_y, m * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    c->F.ncell = (int)nc, c->F.ntr = ntr;
    // zero_wavefield.c, and no source but the residuals (time_loop.c:248-253 with sw = 1)
    if ((rc = sofi_reset(c, -1)))
        return rc;
    // The backward steps write no gradient quantities: they run the variants
    // the autotuner picks for plain steps of this grid (timed now, on the
    // zeroed state, or taken from the cache), the velocity update in its
    // backward form (four, two or one cell per thread on wide blocks, which
    // also injects the residuals and adds the density term); recomputed
    // forward steps run the FWI kernels of the first forward run (fwi_vw, fwi_sw).
    c->fwi_back = true, c->tuned = false;
    rc = autotune(c);
    const int bvw = c->vw, bvrows = 1, bsw = c->sw;
    const bool bvnarrow = false, bsnarrow = c->snarrow;
    c->fwi_back = false;
    if (rc)
        return rc;
    CK(cudaMemsetAsync(c->F.px, 0, n * sizeof(float), c->stream));
    CK(cudaMemsetAsync(c->F.py, 0, n * sizeof(float), c->stream));
    const Acq saved = c->A;
    const bool saved_force = c->has_force;
    auto backward_mode = [&](bool on) {
        if (on) {
            c->A.src_off = c->d_noacq, c->A.last_type = c->d_noacq, c->has_force = false;
            c->vw = bvw, c->vrows = bvrows, c->sw = bsw, c->vnarrow = bvnarrow, c->snarrow = bsnarrow;
        } else {
            c->A = saved, c->has_force = saved_force;
            c->vw = c->fwi_vw, c->vrows = 1, c->sw = c->fwi_sw, c->vnarrow = c->snarrow = false;
        }
        c->fwi_back = on, c->graph_dirty = true;
    };
    if (!c->fwi_K) {
        backward_mode(true);
        rc = sofi_run(c, NT);
    } else {
        // segments last to first: recompute the segment's forward steps from
        // its checkpoint into the store, then run the backward steps that read them
        const int K = c->fwi_K;
        int done = 0;
        for (int seg = c->fwi_nseg - 1; seg >= 0 && !rc; seg--) {
            const int s0 = seg * K, k = std::min(K, NT - s0);
            if (done)
                rc = fwi_copy_state(c, c->fwi_tmp, true);
            if (!rc)
                rc = fwi_copy_state(c, seg ? c->fwi_ckpt + (size_t)(seg - 1) * c->fwi_state : nullptr, false);
            if (!rc)
                rc = fwi_set_step(c, s0, s0);
            if (rc)
                break;
            backward_mode(false);
            c->fwi_store_on = true, c->fwi_nosnap = true;
            // a recomputed segment records no seismograms: the sections keep
            // the backward run's samples, as after a whole-store pass
            c->G.seismo = 0;
            rc = sofi_run(c, k);
            c->G.seismo = c->cfg.seismo;
            if (rc)
                break;
            if ((rc = fwi_copy_state(c, done ? c->fwi_tmp : nullptr, false)) || (rc = fwi_set_step(c, done, s0)))
                break;
            backward_mode(true);
            rc = sofi_run(c, k);
            done += k;
        }
        c->fwi_store_on = false, c->fwi_nosnap = false;
    }
    if (!rc)
        rc = sofi_synchronize(c);
    backward_mode(false);
    return rc;
}

int sofi_fwi_checkpoints(sofi_ctx *c, int *interval, int *segments)
{
    if (!c || !interval || !segments)
        return fail(SOFI_E_ARG, "null argument");
    if (!c->fwi)
        return fail(SOFI_E_STATE, "sofi_fwi_begin first");
    *interval = c->fwi_K, *segments = c->fwi_nseg;
    return 0;
}

int sofi_fwi_gradients(sofi_ctx *c, float *lam, float *mu, float *rhos)
{
    if (!c || !lam || !mu || !rhos)
        return fail(SOFI_E_ARG, "null argument");
    if (!c->fwi)
        return fail(SOFI_E_STATE, "sofi_fwi_begin first");
    CK(cudaSetDevice(c->device));
    const size_t b = (size_t)c->cfg.nx * c->cfg.ny * sizeof(float);
    CK(cudaMemcpyAsync(lam, c->F.g_lam, b, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(mu, c->F.g_mu, b, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(rhos, c->F.g_rhos, b, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int sofi_pdl(sofi_ctx *c, int *on)
{
    if (!c || !on)
        return fail(SOFI_E_ARG, "null argument");
    *on = c->pdl ? 1 : 0;
    return 0;
}

int sofi_set_pdl(sofi_ctx *c, int on)
{
    if (!c)
        return fail(SOFI_E_ARG, "null context");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    c->pdl = on != 0;
    c->graph_dirty = true;
    return 0;
}

int sofi_post_fused(sofi_ctx *c, int *on)
{
    if (!c || !on)
        return fail(SOFI_E_ARG, "null argument");
    *on = post_fused(c) ? 1 : 0;
    return 0;
}

int sofi_block_threads_x(sofi_ctx *c, int *velocity, int *stress)
{
    if (!c || !velocity || !stress)
        return fail(SOFI_E_ARG, "null argument");
    const bool ac = c->cfg.weq == SOFI_AC_ISO, visco = is_visco(c->cfg.weq);
    const int kind = kind_of(c->cfg.weq);
    *velocity = (c->vnarrow && c->vw == 4 && !c->G.ab4 && narrow_v_applies(ac, false)) ? 8 : BX;
    *stress = (c->snarrow && c->sw == 4 && !c->G.ab4 && kind != AC && kind != TTI &&
               narrow_s_applies(visco, visco ? c->G.L : 0, false)) ? 8 : BX;
    return 0;
}

int sofi_stress_variant(sofi_ctx *c, int *cells_per_thread)
{
    if (!c || !cells_per_thread)
        return fail(SOFI_E_ARG, "null argument");
    const int sw = c->sw;
    if (c->G.ab4)
        *cells_per_thread = ab4_wide_s(c) ? 4 : 1;
    else
        *cells_per_thread = kind_of(c->cfg.weq) == TTI ? 1 : (sw ? sw : 1);
    return 0;
}

int sofi_launch_count(sofi_ctx *c, long long *launches)
{
    if (!c || !launches)
        return fail(SOFI_E_ARG, "null argument");
    *launches = c->launches;
    return 0;
}

int sofi_current_step(sofi_ctx *c, int *step)
{
    if (!c || !step)
        return fail(SOFI_E_ARG, "null argument");
    *step = c->step;
    return 0;
}

int sofi_num_samples(sofi_ctx *c, int *ns)
{
    if (!c || !ns)
        return fail(SOFI_E_ARG, "null argument");
    *ns = c->cfg.ndt > 0 ? c->cfg.nt / c->cfg.ndt : 0;
    return 0;
}

int sofi_get_section(sofi_ctx *c, int shot, int comp, float *host)
{
    if (!c || !host || shot < 0 || shot >= c->cfg.nshots || comp < 1 || comp > 5)
        return fail(SOFI_E_ARG, "invalid section arguments");
    CK(cudaSetDevice(c->device));
    if (c->acq_dirty) {
        int rc = upload_acq(c);
        if (rc)
            return rc;
    }
    int rc = sofi_synchronize(c);
    if (rc)
        return rc;
    int r0 = 0;
    for (int s = 0; s < shot; s++)
        r0 += (int)c->acq[s].rix.size();
    int ntr = (int)c->acq[shot].rix.size(), ns = c->A.ns;
    if (!ntr || !ns)
        return 0;
    CK(cudaMemcpy2DAsync(host, sizeof(float) * ns, c->d_sec + ((size_t)r0 * 5 + (comp - 1)) * ns,
                         sizeof(float) * 5 * ns, sizeof(float) * ns, ntr, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int sofi_get_field(sofi_ctx *c, int shot, const char *name, float *host)
{
    if (!c || !name || !host || shot < 0 || shot >= c->cfg.nshots)
        return fail(SOFI_E_ARG, "invalid field arguments");
    CK(cudaSetDevice(c->device));
    float *p = field_ptr(c, shot, name);
    if (!p)
        return fail(SOFI_E_ARG, "unknown wavefield '%s'", name);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy2DAsync(host, sizeof(float) * c->cfg.nx, p + (long long)HY * c->G.pitch + HX,
                         sizeof(float) * c->G.pitch, sizeof(float) * c->cfg.nx, c->cfg.ny, cudaMemcpyDeviceToHost,
                         c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int sofi_set_field(sofi_ctx *c, int shot, const char *name, const float *host)
{
    if (c)
        c->pristine = false;
    if (!c || !name || !host || shot < 0 || shot >= c->cfg.nshots)
        return fail(SOFI_E_ARG, "invalid field arguments");
    CK(cudaSetDevice(c->device));
    float *p = field_ptr(c, shot, name);
    if (!p)
        return fail(SOFI_E_ARG, "unknown wavefield '%s'", name);
    return copy_2d_in(c, p, host, c->cfg.nx, 1);
}

int sofi_num_snapshots(sofi_ctx *c, int *count, int *frame_size)
{
    if (!c)
        return fail(SOFI_E_ARG, "null context");
    if (count)
        *count = c->nsnap;
    if (frame_size)
        *frame_size = c->snap_nx * c->snap_ny;
    return 0;
}

int sofi_get_snapshot(sofi_ctx *c, int shot, int k, int comp, float *host)
{
    if (!c || !host || shot < 0 || shot >= c->cfg.nshots || k < 0 || k >= c->nsnap || comp < 1 || comp > 5)
        return fail(SOFI_E_ARG, "invalid snapshot arguments");
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    long long n = (long long)c->snap_nx * c->snap_ny;
    const float *src = c->d_snap + (long long)shot * n * 5 * c->snap_total + ((long long)k * 5 + (comp - 1)) * n;
    CK(cudaMemcpyAsync(host, src, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int sofi_last_run_ms(sofi_ctx *c, float *ms)
{
    if (!c || !ms)
        return fail(SOFI_E_ARG, "null argument");
    int rc = sofi_synchronize(c);
    *ms = c->last_ms;
    return rc;
}

// ---- allocation-free TTI stress update ------------------------------------
//
// The derivative fields of the TTI stress update (raw and CPML-stretched, 4
// each) live here for sofi_tti_stress_noalloc: a fixed array that every GPU
// loading the library holds until exit, so the entry point needs no
// cudaMalloc. Host code must not use this name as a device address: it looks
// the address up with cudaGetSymbolAddress once per device.
static __device__ __align__(256) float g_noalloc_scratch[8 * SOFI_NOALLOC_MAX_CELLS];

namespace {
constexpr int kMaxDevices = 64;
float *g_noalloc_ptr[kMaxDevices] = {};
std::mutex g_noalloc_mu;  // first calls from several host threads look the address up once
}  // namespace

int sofi_tti_stress_noalloc(const sofi_config *cfg, const sofi_tti_stress_args *a, void *stream)
{
    if (!cfg || !a)
        return fail(SOFI_E_ARG, "null argument");
    if (cfg->weq != SOFI_EL_TTI && cfg->weq != SOFI_VEL_TTI)
        return fail(SOFI_E_ARG, "sofi_tti_stress_noalloc: WEQ must be EL_TTI or VEL_TTI (got %d)", cfg->weq);
    sofi_config c1 = *cfg;
    c1.nshots = 1;
    c1.seismo = 0;
    c1.snap = 0;
    int rc = check_config(&c1);
    if (rc)
        return rc;
    int pitch = pitch_for(cfg->nx);
    long long fsz = (long long)pitch * (cfg->ny + 2 * HY);
    if (fsz > SOFI_NOALLOC_MAX_CELLS)
        return fail(SOFI_E_ARG,
                    "sofi_tti_stress_noalloc: padded grid of %lld cells exceeds the fixed scratch of %ld cells "
                    "(NX %d x NY %d pads to %d x %d)",
                    fsz, (long)SOFI_NOALLOC_MAX_CELLS, cfg->nx, cfg->ny, pitch, cfg->ny + 2 * HY);
    bool visco = cfg->weq == SOFI_VEL_TTI;
    int abs_type = cfg->fw > 0 ? cfg->abs_type : 0;
    if (!a->vx || !a->vy || !a->sxx || !a->syy || !a->sxy || !a->c11 || !a->c13 || !a->c33 || !a->c15 || !a->c35 ||
        !a->c55ipjp || !a->c15ipjp || !a->c35ipjp)
        return fail(SOFI_E_ARG, "sofi_tti_stress_noalloc: a wavefield or modulus pointer is NULL");
    if (visco && (!a->r || !a->p || !a->q || !a->c11d_base || !a->c13d_base || !a->c33d_base || !a->c15d_base ||
                  !a->c35d_base || !a->c55ipjpd_base || !a->c15ipjpd_base || !a->c35ipjpd_base))
        return fail(SOFI_E_ARG, "sofi_tti_stress_noalloc: VEL_TTI needs memory variables and defect bases");
    if (abs_type == 1 && (!a->psi_vxx || !a->psi_vyx || !a->psi_vyy || !a->psi_vxy || !a->K_x || !a->a_x ||
                          !a->b_x || !a->K_x_half || !a->a_x_half || !a->b_x_half || !a->K_y || !a->a_y ||
                          !a->b_y || !a->K_y_half || !a->a_y_half || !a->b_y_half))
        return fail(SOFI_E_ARG, "sofi_tti_stress_noalloc: CPML needs psi memory and profiles");
    if (abs_type == 2 && !a->absorb)
        return fail(SOFI_E_ARG, "sofi_tti_stress_noalloc: damping frame needs absorb");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(SOFI_E_ARG, "device %d beyond the %d the scratch table covers", dev, kMaxDevices);
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_noalloc_ptr[dev] = static_cast<float *>(p);
        }
        scratch = g_noalloc_ptr[dev];
    }
    Geo G{};
    G.nx = cfg->nx, G.ny = cfg->ny, G.pitch = pitch, G.nshots = 1, G.fsz = fsz;
    G.fw = cfg->fw, G.fw2 = 2 * cfg->fw, G.abs_type = abs_type;
    G.free_surf = cfg->free_surf, G.boundary = cfg->boundary, G.L = visco ? cfg->L : 0;
    G.model_stride_on = 0, G.el_tti_rb_short = (cfg->weq == SOFI_EL_TTI);
    int fw = abs_type ? cfg->fw : 0;
    G.gx2 = fw, G.gx3 = cfg->nx - fw, G.gy2 = fw, G.gy3 = cfg->ny - fw;
    if (cfg->free_surf)
        G.gy2 = 0;
    if (cfg->boundary)
        G.gx2 = 0, G.gx3 = cfg->nx;
    G.dt = cfg->dt, G.dh = cfg->dh, G.dtdh = cfg->dt / cfg->dh, G.dhi = 1.0f / cfg->dh, G.dthalbe = cfg->dt / 2.0f;
    for (int k = 0; k < 7; k++)
        G.hc[k] = a->hc[k];
    Wave W{};
    W.vx = const_cast<float *>(a->vx), W.vy = const_cast<float *>(a->vy);
    W.sxx = a->sxx, W.syy = a->syy, W.sxy = a->sxy, W.r = a->r, W.p = a->p, W.q = a->q;
    W.psi_vxx = a->psi_vxx, W.psi_vyx = a->psi_vyx, W.psi_vyy = a->psi_vyy, W.psi_vxy = a->psi_vxy;
    W.draw = scratch;
    W.dcor = scratch + 4 * fsz;
    Model M{};
    M.c11 = a->c11, M.c13 = a->c13, M.c33 = a->c33, M.c15 = a->c15, M.c35 = a->c35;
    M.c55ipjp = a->c55ipjp, M.c15ipjp = a->c15ipjp, M.c35ipjp = a->c35ipjp;
    M.c11b = a->c11d_base, M.c13b = a->c13d_base, M.c33b = a->c33d_base, M.c15b = a->c15d_base;
    M.c35b = a->c35d_base, M.c55ipjpb = a->c55ipjpd_base, M.c15ipjpb = a->c15ipjpd_base;
    M.c35ipjpb = a->c35ipjpd_base, M.absorb = a->absorb;
    M.K_x = a->K_x, M.a_x = a->a_x, M.b_x = a->b_x, M.K_x_half = a->K_x_half, M.a_x_half = a->a_x_half;
    M.b_x_half = a->b_x_half, M.K_y = a->K_y, M.a_y = a->a_y, M.b_y = a->b_y, M.K_y_half = a->K_y_half;
    M.a_y_half = a->a_y_half, M.b_y_half = a->b_y_half;
    for (int l = 0; l < G.L; l++)
        M.bip[l] = a->bip[l], M.cip[l] = a->cip[l], M.peta[l] = a->peta[l];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grd((cfg->nx + BX - 1) / BX, (cfg->ny + BY - 1) / BY, 1);
    launch_tti_split(G, W, M, cfg->fdorder / 2, visco, grd, st);
    CK(cudaGetLastError());
    return 0;
}

}  // extern "C"
