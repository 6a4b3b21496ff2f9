// knc_api.cu — host runtime behind include/knc.h.
//
// Owns the device state of one simulation and sequences the stage kernels.
// It restates the orchestration of src/scheme.rs:212-240 (advance: dt once,
// then `fold` x {add_remove_blocks, RK step}), the RK driver of
// godunov_core::runge_kutta (Shu-Osher forms, b = 1/2; 3/4 then 1/3) and the
// State bookkeeping of src/state.rs (time and Rational64 iteration averaged
// with the same weights as the conserved data). Geometry tables follow
// src/mesh.rs:119-407 and are computed here once per block.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "knc_internal.h"
#include "knc_tma.cuh"

using namespace knc;

namespace {

constexpr double PI_H = 3.14159265358979323846;
constexpr double LIGHT_SPEED_H = 3e10;

// ---------------------------------------------------------------- geometry --
struct ExtentH { double r0, r1, q0, q1; };

struct MeshH {
    knc_mesh_params p;
    double zone_dlogr() const {                                   // mesh.rs:341-346
        return p.has_num_radial_zones ? 1.0 / (double)p.num_radial_zones : PI_H / (double)p.num_polar_zones;
    }
    double block_dlogr() const { return (double)p.block_size * zone_dlogr(); }
    ExtentH extent(int32_t index) const {                         // mesh.rs:358-372
        double q0 = 0.0, q1 = PI_H;
        if (p.num_polar_zones == 1) { q0 = PI_H * 0.5 - zone_dlogr(); q1 = PI_H * 0.5 + zone_dlogr(); }
        ExtentH e;
        e.r0 = p.reference_radius * std::pow(1.0 + block_dlogr(), (double)index);
        e.r1 = p.reference_radius * std::pow(1.0 + block_dlogr(), (double)index + 1.0);
        e.q0 = q0;
        e.q1 = q1;
        return e;
    }
    double t_start() const { return p.has_excision_delay ? p.excision_delay : 0.0; }
    double ies(double t) const { return p.inner_radius + std::max(t - t_start(), 0.0) * p.inner_excision_speed; }
    double oes(double t) const { return p.outer_radius + std::max(t - t_start(), 0.0) * p.outer_excision_speed; }
    bool moving() const { return p.inner_excision_speed > 0.0 || p.outer_excision_speed > 0.0; }
};

// SphericalPolarGrid::vertex_coordinate_signed (mesh.rs:202-210); Rust's
// f64::log(base) is ln(x) / ln(base).
double vertex_r(const ExtentH& e, int64_t nr, int64_t i) {
    const double y0 = std::log(e.r0) / std::log(10.0);
    const double y1 = std::log(e.r1) / std::log(10.0);
    const double dy = (y1 - y0) / (double)nr;
    return std::pow(10.0, y0 + dy * (double)i);
}
double vertex_q(const ExtentH& e, int64_t nq, int64_t j) {
    const double dq = (e.q1 - e.q0) / (double)nq;
    return e.q0 + dq * (double)j;
}
double cell_volume(double r0, double q0, double r1, double q1) {            // mesh.rs:119-123
    const double dcost = -(std::cos(q1) - std::cos(q0));
    return 2.0 * PI_H * (r1 * r1 * r1 - r0 * r0 * r0) / 3.0 * dcost;
}
double face_area(double r0, double q0, double r1, double q1) {              // mesh.rs:125-134
    const double s0 = r0 * std::sin(q0);
    const double s1 = r1 * std::sin(q1);
    const double z0 = r0 * std::cos(q0);
    const double z1 = r1 * std::cos(q1);
    const double ds = s1 - s0;
    const double dz = z1 - z0;
    return PI_H * (s0 + s1) * std::sqrt(ds * ds + dz * dz);
}

struct GeomH {
    int64_t nr = 0, nq = 0;
    std::vector<double> rv, qv, ar, aq, dv, rc, qc, cot;
    std::vector<float2> ar_r, ar_q, aq_r, aq_q, dv_r, dv_q;
    std::vector<float> dv_r32, rc32, cot32;
};

// x as an unevaluated pair of floats hi + lo (|lo| <= ulp(hi) / 2).
float2 split_df(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// Length unit L = 2^e of the mixed stage's FP32 geometry: the power of two at
// or below the reference radius, so FP32 radii stay near 1 whatever the
// units (code units: e = 0; the reference's cgs setups: r ~ 1e8-1e19 cm, where
// c r^3 in cm^3 cm/s would overflow FP32).
int length_exponent(const knc_mesh_params& p) {
    int e = 0;
    std::frexp(p.reference_radius, &e);
    return e - 1;
}

GeomH make_geometry(const MeshH& M, int32_t index, bool with_faces = true, double cflux = 1.0, int64_t nr = 0,
                    int64_t nq = 0) {   // mesh.rs:246-264
    GeomH G;
    const ExtentH e = M.extent(index);
    if (nr <= 0) nr = M.p.block_size;
    if (nq <= 0) nq = M.p.num_polar_zones;
    G.nr = nr;
    G.nq = nq;
    G.rv.resize(nr + 1);
    G.qv.resize(nq + 1);
    for (int64_t i = 0; i <= nr; ++i) G.rv[i] = vertex_r(e, nr, i);
    for (int64_t j = 0; j <= nq; ++j) G.qv[j] = vertex_q(e, nq, j);
    G.dv.resize(nr * nq);
    G.rc.resize(nr);
    G.qc.resize(nq);
    G.cot.resize(nq);
    for (int64_t i = 0; i < nr; ++i) {
        G.rc[i] = std::sqrt(G.rv[i] * G.rv[i + 1]);                              // mesh.rs:157-161
        for (int64_t j = 0; j < nq; ++j)
            G.dv[i * nq + j] = cell_volume(G.rv[i], G.qv[j], G.rv[i + 1], G.qv[j + 1]);
    }
    for (int64_t j = 0; j < nq; ++j) {
        G.qc[j] = 0.5 * (G.qv[j] + G.qv[j + 1]);
        G.cot[j] = std::cos(G.qc[j]) / std::sin(G.qc[j]);
    }
    if (!with_faces) return G;
    G.ar.resize((nr + 1) * nq);
    G.aq.resize(nr * (nq + 1));
    for (int64_t i = 0; i <= nr; ++i)
        for (int64_t j = 0; j < nq; ++j) G.ar[i * nq + j] = face_area(G.rv[i], G.qv[j], G.rv[i], G.qv[j + 1]);
    for (int64_t i = 0; i < nr; ++i)
        for (int64_t j = 0; j <= nq; ++j)
            G.aq[i * (nq + 1) + j] = face_area(G.rv[i], G.qv[j], G.rv[i + 1], G.qv[j]);
    // separable factors for the mixed path (double-float pairs, c folded in),
    // lengths in units of L = 2^e (exact power-of-two scalings)
    const int le = length_exponent(M.p);
    G.ar_r.resize(nr + 1);
    G.aq_r.resize(nr);
    G.dv_r.resize(nr);
    G.dv_r32.resize(nr);
    G.rc32.resize(nr);
    for (int64_t i = 0; i <= nr; ++i) G.ar_r[i] = split_df(std::ldexp(cflux * (G.rv[i] * G.rv[i]), -2 * le));
    for (int64_t i = 0; i < nr; ++i) {
        const double a = G.rv[i], b = G.rv[i + 1];
        G.aq_r[i] = split_df(std::ldexp(cflux * (PI_H * (b * b - a * a)), -2 * le));
        const double v = (b * b * b - a * a * a) * 2.0 * PI_H / 3.0;
        G.dv_r[i] = split_df(std::ldexp(cflux * v, -3 * le));
        G.dv_r32[i] = (float)std::ldexp(v, -3 * le);
        G.rc32[i] = (float)std::ldexp(G.rc[i], -le);
    }
    G.ar_q.resize(nq);
    G.aq_q.resize(nq + 1);
    G.dv_q.resize(nq);
    G.cot32.resize(nq);
    for (int64_t j = 0; j < nq; ++j) {
        const double s0 = std::sin(G.qv[j]), s1 = std::sin(G.qv[j + 1]);
        const double c0 = std::cos(G.qv[j]), c1 = std::cos(G.qv[j + 1]);
        G.ar_q[j] = split_df(PI_H * (s0 + s1) * std::sqrt((s1 - s0) * (s1 - s0) + (c1 - c0) * (c1 - c0)));
        G.dv_q[j] = split_df(c0 - c1);
        G.cot32[j] = (float)G.cot[j];
    }
    for (int64_t j = 0; j <= nq; ++j) G.aq_q[j] = split_df(std::sin(G.qv[j]));
    return G;
}

// ---------------------------------------------------------------- helpers --
struct Rational {
    int64_t n = 0, d = 1;
    static int64_t gcd(int64_t a, int64_t b) {
        if (a < 0) a = -a;
        if (b < 0) b = -b;
        while (b) { const int64_t t = a % b; a = b; b = t; }
        return a ? a : 1;
    }
    void norm() { const int64_t g = gcd(n, d); n /= g; d /= g; if (d < 0) { n = -n; d = -d; } }
    Rational add(const Rational& o) const { Rational r; r.n = n * o.d + o.n * d; r.d = d * o.d; r.norm(); return r; }
    Rational mul(const Rational& o) const { Rational r; r.n = n * o.n; r.d = d * o.d; r.norm(); return r; }
};

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    if (count == 0) { *p = nullptr; return cudaSuccess; }
    return cudaMalloc((void**)p, count * sizeof(T));
}
template <class T>
cudaError_t upload(T** p, const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = dalloc(p, v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

struct BlockH {
    int32_t index = 0;
    int64_t nr = 0, nq = 0;
    double* buf[2] = {nullptr, nullptr};
    void* P = nullptr;
    double* P64 = nullptr;   // mixed stage: FP64 primitives of the zones above the split
    double *ar = nullptr, *aq = nullptr, *dv = nullptr, *rc = nullptr, *rv = nullptr;
    float2 *ar_r = nullptr, *aq_r = nullptr, *dv_r = nullptr;
    float *dv_r32 = nullptr, *rc32 = nullptr;
    GeomH geom;   // host copy (rc, qc for error positions; dv for error values)
};

void free_block(BlockH& b) {
    cudaFree(b.buf[0]);
    cudaFree(b.buf[1]);
    cudaFree(b.P);
    cudaFree(b.P64);
    cudaFree(b.ar);
    cudaFree(b.aq);
    cudaFree(b.dv);
    cudaFree(b.rc);
    cudaFree(b.rv);
    cudaFree(b.ar_r);
    cudaFree(b.aq_r);
    cudaFree(b.dv_r);
    cudaFree(b.dv_r32);
    cudaFree(b.rc32);
    b = BlockH();
}

// Rows of the warp strips the host-state advance updates chunks with
// (host-state step on the 4096 x 1024 wind: 2, 4, 8 rows measured 1.372,
// 1.358, 1.379 ms).
constexpr int STREAM_STRIP_ROWS = 4;

// One block set's device view.
struct Layout {
    DevBlock* d_table = nullptr;
    int table_cap = 0;
    int4* d_tiles = nullptr;
    int tiles_cap = 0;
    int ntiles = 0;
    int4* d_utiles = nullptr;   // update tiles of `utr` rows
    int utiles_cap = 0;
    int nutiles = 0;
    int utr = 0;
    int uform = -1;
    int64_t nzones = 0;         // zones of the block set
    TmaMaps* d_tmaps = nullptr; // tensor maps per slot (tiles of `utr` rows), when every block allows them
    int tmaps_cap = 0;
    bool tma_ok = false;
    int4* d_strips = nullptr;   // warp strips {slot, i0, j0, rows} of `utr` rows (strip form)
    int strips_cap = 0;
    int nstrips = 0;
    int chunk_nt = 0;           // zones per fused recovery chunk (= fused CTA threads)
    int4* d_chunks = nullptr;   // fused recovery chunks {slot, z0, nz, 0} of <= stage_threads(utr) zones
    int chunks_cap = 0;
    int nchunks = 0;
    // halo remaps across polar-resolution changes
    int4* d_remap = nullptr;
    int remap_cap = 0;
    int nremap = 0;
    int max_nq = 0;
    std::vector<int32_t> slot_index;   // slot -> block index
    // per slot (and one past the last): its first recovery tile, update tile,
    // warp strip and zone in the flat whole-state order; the lists hold the
    // blocks in slot order, so a run of slots is a run of each list
    std::vector<int> tile_off, utile_off, strip_off, sstrip_off;
    std::vector<int64_t> zone_off;
    // warp strips of STREAM_STRIP_ROWS rows for the host-state advance, whose
    // launches each cover one chunk of blocks: short strips keep enough
    // warps per SM on a chunk
    int4* d_sstrips = nullptr;
    int sstrips_cap = 0;
    std::vector<DevBlock> tab_h;   // host copies of d_table, d_tiles and d_sstrips
    std::vector<int4> tiles_h, sstrips_h;
    // the host-state advance's independent chunks, built for sc_S stages on
    // first use (build_chunks): a table with shadow blocks appended, per chunk
    // its recovery tiles (own blocks' first) and per chunk and stage its strips
    int sc_S = 0;
    std::vector<int> sc_cb;              // [G + 1] chunk bounds (slots)
    std::vector<int> sc_tile_off;        // [G + 1]
    std::vector<int> sc_own_tiles;       // [G]
    std::vector<int> sc_strip_off;       // [G S + 1]: chunk k, stage s at k S + s
    std::vector<int64_t> sc_up;          // [G + 1]: zones each chunk's upload covers
    DevBlock* d_sc_table = nullptr;
    int sc_table_cap = 0;
    int4* d_sc_tiles = nullptr;
    int sc_tiles_cap = 0;
    int4* d_sc_strips = nullptr;
    int sc_strips_cap = 0;
    double* d_sc_store = nullptr;
    size_t sc_store_cap = 0;
    // edge blocks, whose outer halo rows the ghost launch writes
    void* P_edge[2] = {nullptr, nullptr};
    double* P64_edge[2] = {nullptr, nullptr};
    int32_t nr_edge[2] = {0, 0}, nq_edge[2] = {0, 0};
    // ghost rows
    int32_t ghost_lo = INT32_MIN, ghost_hi = INT32_MIN;
    double* d_ghost_rc = nullptr;                  // [2 ends][2 rows]
    double* d_ghost_dv[2] = {nullptr, nullptr};    // per end [2][nq]
    int64_t ghost_nq[2] = {0, 0};
    std::vector<double> ghost_rc_h, ghost_dv_h[2];
    // a block activated at the start of the step this layout begins
    int4* d_init_tiles = nullptr;
    int n_init_tiles = 0;
    int32_t first_stage = 0;   // stage counter when the layout took effect
};

void free_layout(Layout& l) {
    cudaFree(l.d_table);
    cudaFree(l.d_tiles);
    cudaFree(l.d_utiles);
    cudaFree(l.d_chunks);
    cudaFree(l.d_strips);
    cudaFree(l.d_sstrips);
    cudaFree(l.d_tmaps);
    cudaFree(l.d_remap);
    cudaFree(l.d_ghost_rc);
    cudaFree(l.d_ghost_dv[0]);
    cudaFree(l.d_ghost_dv[1]);
    cudaFree(l.d_init_tiles);
    cudaFree(l.d_sc_table);
    cudaFree(l.d_sc_tiles);
    cudaFree(l.d_sc_strips);
    cudaFree(l.d_sc_store);
    l = Layout();
}

}  // namespace

struct knc_ctx {
    knc_hydro_params hp{};
    MeshH mesh{};
    knc_model_params model{};
    bool have_model = false;
    knc_primitive_at_fn host_fn = nullptr;
    void* host_user = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;        // ghost rows run here, beside the recovery
    // host-state advance: uploads and downloads of block chunks, beside the stages
    cudaStream_t h2d = nullptr, d2h = nullptr;
    std::vector<cudaStream_t> kstreams;   // one per kind of chunk launch (recovery / update of each stage)
    std::vector<cudaEvent_t> ev_chunk;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::map<int32_t, BlockH> blocks;
    std::map<std::pair<int64_t, int64_t>, std::vector<BlockH>> pool;   // freed block storage by shape
    int cur = 0;
    // uneven blocks: index -> (nr, nq); other indexes use the mesh's shape
    std::map<int32_t, std::pair<int64_t, int64_t>> shapes;
    // per-column tables, one set per polar resolution in use
    struct ColTab {
        double *qv = nullptr, *qc = nullptr, *cot = nullptr;
        float2 *ar_q = nullptr, *aq_q = nullptr, *dv_q = nullptr;
        float* cot32 = nullptr;
        std::vector<double> qc_h;
    };
    std::map<int64_t, ColTab> cols;
    // Device view of a block set (table, tiles, remaps, ghost rows). A
    // captured fold whose excision surfaces move holds one per block set it
    // passes through; otherwise there is one, rebuilt in place.
    std::vector<Layout> lays{1};
    int cur_lay = 0;
    bool dirty = true;
    std::vector<BlockH> deferred;    // retired inside a captured fold, released after it ran
    double* d_host_prim = nullptr;   // host model values
    size_t host_prim_cap = 0;
    // status
    DevStatus* d_status = nullptr;
    DevStatus* h_status = nullptr;
    int32_t stage_counter = 0;
    bool failed = false;
    // time
    double time = 0.0;
    Rational iteration;
    // chosen forms
    int32_t precision = KNC_PRECISION_FP64;
    int32_t guess = KNC_GUESS_PLAIN;
    int32_t batched = 0;
    int32_t utr = 8;   // update tile rows (4, 8 or 16)
    int32_t fused = 0;         // one cooperative launch per stage
    int32_t uform = KNC_UPDATE_TILE;   // update form of the separate stage
    int32_t rform = KNC_RECOVERY_INLINE;   // mixed recovery form of the separate stage
    int32_t ctas_per_sm = 0;   // fused grid: CTAs per SM (0: the occupancy bound)
    int32_t sms = 0;
    bool coop = false;         // the device supports cooperative launches
    unsigned long long bar_epoch = 0;   // grid-barrier arrivals issued since the status reset
    // adaptive dt found on the device in the fold's first recovery, with no
    // separate pass (set by knc_advance for one fold)
    bool ddt = false;
    double ddt_t0 = 0.0;   // time at the start of the fold
    int ddt_step = 0;      // step of the fold being issued
    double w_split = 2.0;
    float* d_mlp = nullptr;
    // stage lists shared by every layout (rebuild_table grows them)
    int2* d_high = nullptr;     // mixed recovery: zones deferred to the dense FP64 pass
    int64_t high_cap = 0;
    int2* d_hp = nullptr;       // mixed stage: stored zones above the Lorentz-factor split (drain_hp)
    int64_t hp_cap = 0;
    // the bounded-wait test (knc_set_wait_test): poll limit of the fused
    // stage's grid barriers (0: the default) and a barrier that cannot complete
    int32_t wait_polls = 0;
    int32_t wait_unreachable = 0;
    // bookkeeping
    int64_t launches = 0;
    int64_t zone_updates = 0;   // zones x RK steps advanced since creation
    bool profiling = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_events;
    std::vector<cudaEvent_t> event_pool;
    double prof_ms[KNC_KERNEL_KINDS] = {};
    int64_t prof_count[KNC_KERNEL_KINDS] = {};
    bool capturing = false;
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t marks[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    knc_error err{};
    double* d_stage = nullptr;
    size_t stage_cap = 0;
};

namespace {

inline Layout& L(knc_ctx* c) { return c->lays[c->cur_lay]; }
inline const Layout& L(const knc_ctx* c) { return c->lays[c->cur_lay]; }

int set_msg(knc_ctx* c, int status, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
int set_msg(knc_ctx* c, int status, const char* fmt, ...) {
    if (!c) return status;
    std::memset(&c->err, 0, sizeof(c->err));
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(c->err.message, sizeof(c->err.message), fmt, ap);
    va_end(ap);
    return status;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            if (e_ == cudaErrorMemoryAllocation)                                                   \
                return set_msg(c, KNC_ERR_OUT_OF_MEMORY, "%s: %s", #call, cudaGetErrorString(e_)); \
            return set_msg(c, KNC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));               \
        }                                                                                          \
    } while (0)

int validate(knc_ctx* c, const knc_hydro_params* h, const knc_mesh_params* m) {
    if (h->system != KNC_SYSTEM_RELATIVISTIC && h->system != KNC_SYSTEM_NEWTONIAN)
        return set_msg(c, KNC_ERR_CONFIG, "unknown hydro system %d", h->system);
    if (h->plm_theta < 1.0 || h->plm_theta > 2.0)
        return set_msg(c, KNC_ERR_CONFIG, "plm_theta must be in the range [1, 2]");
    if (h->cfl_number < 0.0 || h->cfl_number > 0.7)
        return set_msg(c, KNC_ERR_CONFIG, "cfl_number must be in the range [0.0, 0.7]");
    if (h->runge_kutta_order < 1 || h->runge_kutta_order > 3)
        return set_msg(c, KNC_ERR_CONFIG, "runge_kutta_order must be RK1, RK2 or RK3");
    if (h->riemann_solver != KNC_RIEMANN_HLLE && h->riemann_solver != KNC_RIEMANN_HLLC)
        return set_msg(c, KNC_ERR_CONFIG, "unknown riemann solver");
    if (!(h->gamma_law_index > 1.0)) return set_msg(c, KNC_ERR_CONFIG, "gamma_law_index must exceed 1");
    if (m->reference_radius <= 0.0 || m->inner_radius < 0.0 || m->outer_radius < 0.0)
        return set_msg(c, KNC_ERR_CONFIG, "all radii must be positive");
    // the reference radius against the outer excision surface depends on the
    // start time (Mesh::validate(time), src/mesh.rs:277-279): checked by
    // knc_init_from_model, which knows the time
    if (m->has_excision_delay && m->excision_delay < 0.0)
        return set_msg(c, KNC_ERR_CONFIG, "the excision delay time must be non-negative");
    if (m->inner_excision_speed < 0.0 || m->outer_excision_speed < 0.0)
        return set_msg(c, KNC_ERR_CONFIG, "the excision surface speeds must be non-negative");
    if (m->outer_excision_speed < m->inner_excision_speed)
        return set_msg(c, KNC_ERR_CONFIG, "outer_excision_speed < inner_excision_speed");
    if (m->block_size < 2) return set_msg(c, KNC_ERR_CONFIG, "must have at least 2 radial zones per block");
    if (m->num_polar_zones != 1 && m->num_polar_zones < 16)
        return set_msg(c, KNC_ERR_CONFIG, "must have at least 16 polar zones");
    if (m->num_polar_zones == 1 && !m->has_num_radial_zones)
        return set_msg(c, KNC_ERR_CONFIG, "num_radial_zones is not optional when num_polar_zones=1");
    if (m->block_size > 16383 || m->num_polar_zones > 65535)
        return set_msg(c, KNC_ERR_CONFIG, "block shape exceeds 16383 x 65535");
    return KNC_OK;
}

std::pair<int64_t, int64_t> shape_of(const knc_ctx* c, int32_t index) {
    auto it = c->shapes.find(index);
    if (it != c->shapes.end()) return it->second;
    return {c->mesh.p.block_size, c->mesh.p.num_polar_zones};
}

double cflux_of(const knc_ctx* c) { return c->hp.system == KNC_SYSTEM_RELATIVISTIC ? LIGHT_SPEED_H : 1.0; }

// Column tables of a polar resolution, built on first use.
int get_cols(knc_ctx* c, int64_t nq, knc_ctx::ColTab** out) {
    auto it = c->cols.find(nq);
    if (it == c->cols.end()) {
        const GeomH G = make_geometry(c->mesh, 0, true, cflux_of(c), 2, nq);
        knc_ctx::ColTab t;
        cudaStream_t s = c->stream;
        CK(upload(&t.qv, G.qv, s));
        CK(upload(&t.qc, G.qc, s));
        CK(upload(&t.cot, G.cot, s));
        CK(upload(&t.ar_q, G.ar_q, s));
        CK(upload(&t.aq_q, G.aq_q, s));
        CK(upload(&t.dv_q, G.dv_q, s));
        CK(upload(&t.cot32, G.cot32, s));
        CK(cudaStreamSynchronize(s));
        t.qc_h = G.qc;
        it = c->cols.emplace(nq, t).first;
    }
    *out = &it->second;
    return KNC_OK;
}

int alloc_block(knc_ctx* c, int32_t index, BlockH& b) {
    const auto shape = shape_of(c, index);
    const int64_t nr = shape.first, nq = shape.second;
    auto key = std::make_pair(nr, nq);
    auto it = c->pool.find(key);
    b.geom = make_geometry(c->mesh, index, true, cflux_of(c), nr, nq);
    b.index = index;
    b.nr = nr;
    b.nq = nq;
    if (it != c->pool.end() && !it->second.empty()) {
        BlockH r = it->second.back();
        it->second.pop_back();
        b.buf[0] = r.buf[0];
        b.buf[1] = r.buf[1];
        b.P = r.P;
        b.P64 = r.P64;
        b.ar = r.ar;
        b.aq = r.aq;
        b.dv = r.dv;
        b.rc = r.rc;
        b.rv = r.rv;
        b.ar_r = r.ar_r;
        b.aq_r = r.aq_r;
        b.dv_r = r.dv_r;
        b.dv_r32 = r.dv_r32;
        b.rc32 = r.rc32;
    } else {
        const size_t n = (size_t)(nr * nq);
        CK(dalloc(&b.buf[0], 5 * n));
        CK(dalloc(&b.buf[1], 5 * n));
        CK(cudaMalloc(&b.P, 5 * (size_t)((nr + 4) * nq) * sizeof(double)));
        CK(dalloc(&b.P64, 5 * (size_t)((nr + 4) * nq)));
        CK(dalloc(&b.ar, (size_t)((nr + 1) * nq)));
        CK(dalloc(&b.aq, (size_t)(nr * (nq + 1))));
        CK(dalloc(&b.dv, n));
        CK(dalloc(&b.rc, (size_t)nr));
        CK(dalloc(&b.rv, (size_t)nr + 1));
        CK(dalloc(&b.ar_r, (size_t)nr + 1));
        CK(dalloc(&b.aq_r, (size_t)nr));
        CK(dalloc(&b.dv_r, (size_t)nr));
        CK(dalloc(&b.dv_r32, (size_t)nr));
        CK(dalloc(&b.rc32, (size_t)nr));
    }
    const GeomH& G = b.geom;
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(b.ar, G.ar.data(), G.ar.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.aq, G.aq.data(), G.aq.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.dv, G.dv.data(), G.dv.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.rc, G.rc.data(), G.rc.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.rv, G.rv.data(), G.rv.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.ar_r, G.ar_r.data(), G.ar_r.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.aq_r, G.aq_r.data(), G.aq_r.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.dv_r, G.dv_r.data(), G.dv_r.size() * 8, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.dv_r32, G.dv_r32.data(), G.dv_r32.size() * 4, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(b.rc32, G.rc32.data(), G.rc32.size() * 4, cudaMemcpyHostToDevice, s));
    // host geometry vectors are only needed for positions, volumes, ghosts
    b.geom.ar.clear();
    b.geom.ar.shrink_to_fit();
    b.geom.aq.clear();
    b.geom.aq.shrink_to_fit();
    // zero the primitive array so halo rows of an edge block start defined
    CK(cudaMemsetAsync(b.P, 0, 5 * (size_t)((b.nr + 4) * b.nq) * sizeof(double), s));
    // the copies above read host vectors that live in `b`; finish them now
    CK(cudaStreamSynchronize(s));
    return KNC_OK;
}

void release_block(knc_ctx* c, BlockH& b) {
    c->pool[std::make_pair(b.nr, b.nq)].push_back(b);
    b = BlockH();
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tensor maps of one block for update tiles of `tr` rows: P as float
// {nq, nr+4, 5} with boxes {TILE_Q+8, tr+4, 5} (the tile, its 2-zone halo and
// a 16-byte-aligned start column j0 - 4), each state buffer as double
// {nq, nr, 5} with boxes {TILE_Q, tr, 5}. Needs rows of 16-byte multiples
// (nq % 4 == 0) and a block at least one box wide.
bool encode_block_maps(const BlockH& b, int tr, TmaMaps* m) {
    auto enc = tensor_map_encoder();
    if (!enc || b.nq % 4 != 0 || b.nq < TILE_Q + 8 || b.nr < tr) return false;
    const cuuint64_t nq = (cuuint64_t)b.nq, nr = (cuuint64_t)b.nr;
    const cuuint32_t es[3] = {1, 1, 1};
    const cuuint64_t dimP[3] = {nq, nr + 4, (cuuint64_t)NFIELD};
    const cuuint64_t strP[2] = {nq * 4, (nr + 4) * nq * 4};
    const cuuint32_t boxP[3] = {(cuuint32_t)(TILE_Q + 8), (cuuint32_t)(tr + 4), (cuuint32_t)NFIELD};
    if (enc(&m->P, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, b.P, dimP, strP, boxP, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const cuuint64_t dimU[3] = {nq, nr, (cuuint64_t)NFIELD};
    const cuuint64_t strU[2] = {nq * 8, nr * nq * 8};
    const cuuint32_t boxU[3] = {(cuuint32_t)TILE_Q, (cuuint32_t)tr, (cuuint32_t)NFIELD};
    for (int k = 0; k < 2; ++k)
        if (enc(&m->U[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, b.buf[k], dimU, strU, boxU, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    return true;
}

// Threads of a fused-stage CTA (and zones of its recovery chunks): the mixed
// strip-only kernel runs CTAs of STRIP_WARPS warps, the others (TR+1) warps.
int fused_threads(const knc_ctx* c) {
    return c->precision == KNC_PRECISION_MIXED && c->uform == KNC_UPDATE_STRIP ? STRIP_WARPS * 32
                                                                              : stage_threads(fused_tr(c->utr));
}

// Rebuild the device block table and the tile list after the block set changed.
int rebuild_table(knc_ctx* c) {
    if (!c->dirty && L(c).utr == c->utr && L(c).uform == c->uform && L(c).chunk_nt == fused_threads(c))
        return KNC_OK;
    const int nb = (int)c->blocks.size();
    std::vector<DevBlock> tab(nb);
    std::vector<int4> tiles, utiles, chunks, strips;
    std::vector<TmaMaps> maps(nb);
    bool tma_ok = nb > 0;
    const int nt = fused_threads(c);
    L(c).slot_index.clear();
    L(c).tile_off.clear();
    L(c).utile_off.clear();
    L(c).strip_off.clear();
    L(c).sstrip_off.clear();
    L(c).zone_off.clear();
    std::vector<int4> sstrips;
    int slot = 0;
    int64_t zoff = 0;
    const BlockH* prev = nullptr;
    std::vector<const BlockH*> order;
    std::vector<int4> remaps;
    L(c).max_nq = 0;
    for (auto& kv : c->blocks) order.push_back(&kv.second);
    for (int k = 0; k < nb; ++k) {
        const BlockH& b = *order[k];
        DevBlock& d = tab[k];
        std::memset(&d, 0, sizeof(d));
        knc_ctx::ColTab* ct = nullptr;
        int r0;
        if ((r0 = get_cols(c, b.nq, &ct))) return r0;
        L(c).max_nq = std::max<int>(L(c).max_nq, (int)b.nq);
        d.buf[0] = b.buf[0];
        d.buf[1] = b.buf[1];
        d.P = b.P;
        d.P64 = b.P64;
        d.ar = b.ar;
        d.aq = b.aq;
        d.dv = b.dv;
        d.rc = b.rc;
        d.rv = b.rv;
        d.qv = ct->qv;
        d.qc = ct->qc;
        d.cot = ct->cot;
        d.ar_r = b.ar_r;
        d.ar_q = ct->ar_q;
        d.aq_r = b.aq_r;
        d.aq_q = ct->aq_q;
        d.dv_r = b.dv_r;
        d.dv_q = ct->dv_q;
        d.dv_r32 = b.dv_r32;
        d.rc32 = b.rc32;
        d.cot32 = ct->cot32;
        d.slot_in = -1;
        d.slot_out = -1;
        d.nr = (int32_t)b.nr;
        d.nq = (int32_t)b.nq;
        d.index = b.index;
        if (prev && prev->index + 1 == b.index) {
            d.slot_in = k - 1;
            tab[k - 1].slot_out = k;
            if (prev->nq == b.nq) {      // same polar grid: the producer pushes halo rows
                d.P_in_nbr = prev->P;
                d.nr_in_nbr = (int32_t)prev->nr;
                tab[k - 1].P_out_nbr = b.P;
                tab[k - 1].nr_out_nbr = (int32_t)b.nr;
            } else {                     // remapped after the recovery pass
                remaps.push_back(make_int4(k, k - 1, 0, 0));
                remaps.push_back(make_int4(k - 1, k, 1, 0));
            }
        }
        L(c).tile_off.push_back((int)tiles.size());
        L(c).utile_off.push_back((int)utiles.size());
        L(c).strip_off.push_back((int)strips.size());
        L(c).sstrip_off.push_back((int)sstrips.size());
        L(c).zone_off.push_back(zoff);
        for (int64_t j0 = 0; j0 < b.nq; j0 += STRIP_OUT)
            for (int64_t i0 = 0; i0 < b.nr; i0 += STREAM_STRIP_ROWS)
                sstrips.push_back(
                    make_int4(slot, (int)i0, (int)j0, (int)std::min<int64_t>(STREAM_STRIP_ROWS, b.nr - i0)));
        for (int64_t i0 = 0; i0 < b.nr; i0 += TILE_R)
            for (int64_t j0 = 0; j0 < b.nq; j0 += TILE_Q)
                tiles.push_back(make_int4(slot, (int)i0, (int)j0, (int)zoff));
        if (c->uform == KNC_UPDATE_STRIP) {
            // ceil(nr / utr) strips per column, their heights as even as
            // whole rows allow (64 rows at utr 13: 13, 13, 13, 13, 12)
            const int64_t per = (b.nr + c->utr - 1) / c->utr;
            for (int64_t j0 = 0; j0 < b.nq; j0 += STRIP_OUT)
                for (int64_t k = 0, i0 = 0; k < per; ++k) {
                    const int64_t rows = b.nr / per + (k < b.nr % per ? 1 : 0);
                    strips.push_back(make_int4(slot, (int)i0, (int)j0, (int)rows));
                    i0 += rows;
                }
        } else {
            for (int64_t i0 = 0; i0 < b.nr; i0 += c->utr)
                for (int64_t j0 = 0; j0 < b.nq; j0 += TILE_Q)
                    utiles.push_back(make_int4(slot, (int)i0, (int)j0, 0));
        }
        if (tma_ok) tma_ok = c->utr <= 16 && encode_block_maps(b, c->utr, &maps[k]);
        for (int64_t z0 = 0; z0 < b.nr * b.nq; z0 += nt)
            chunks.push_back(make_int4(slot, (int)z0, (int)std::min<int64_t>(nt, b.nr * b.nq - z0), 0));
        L(c).slot_index.push_back(b.index);
        zoff += b.nr * b.nq;
        prev = &b;
        ++slot;
    }
    L(c).tile_off.push_back((int)tiles.size());
    L(c).utile_off.push_back((int)utiles.size());
    L(c).strip_off.push_back((int)strips.size());
    L(c).sstrip_off.push_back((int)sstrips.size());
    L(c).zone_off.push_back(zoff);
    if ((int)sstrips.size() > L(c).sstrips_cap) {
        cudaFree(L(c).d_sstrips);
        L(c).d_sstrips = nullptr;
        CK(dalloc(&L(c).d_sstrips, sstrips.size()));
        L(c).sstrips_cap = (int)sstrips.size();
    }
    if (!sstrips.empty())
        CK(cudaMemcpyAsync(L(c).d_sstrips, sstrips.data(), sstrips.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    if (nb > L(c).table_cap) {
        cudaFree(L(c).d_table);
        L(c).d_table = nullptr;
        CK(dalloc(&L(c).d_table, (size_t)nb));
        L(c).table_cap = nb;
    }
    if ((int)tiles.size() > L(c).tiles_cap) {
        cudaFree(L(c).d_tiles);
        L(c).d_tiles = nullptr;
        CK(dalloc(&L(c).d_tiles, tiles.size()));
        L(c).tiles_cap = (int)tiles.size();
    }
    if (nb) CK(cudaMemcpyAsync(L(c).d_table, tab.data(), nb * sizeof(DevBlock), cudaMemcpyHostToDevice, c->stream));
    L(c).tab_h = tab;
    L(c).tiles_h = tiles;
    L(c).sstrips_h = sstrips;
    L(c).sc_S = 0;
    if (!tiles.empty())
        CK(cudaMemcpyAsync(L(c).d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
    if ((int)utiles.size() > L(c).utiles_cap) {
        cudaFree(L(c).d_utiles);
        L(c).d_utiles = nullptr;
        CK(dalloc(&L(c).d_utiles, utiles.size()));
        L(c).utiles_cap = (int)utiles.size();
    }
    if (!utiles.empty())
        CK(cudaMemcpyAsync(L(c).d_utiles, utiles.data(), utiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    L(c).nutiles = (int)utiles.size();
    L(c).utr = c->utr;
    if ((int)chunks.size() > L(c).chunks_cap) {
        cudaFree(L(c).d_chunks);
        L(c).d_chunks = nullptr;
        CK(dalloc(&L(c).d_chunks, chunks.size()));
        L(c).chunks_cap = (int)chunks.size();
    }
    if (!chunks.empty())
        CK(cudaMemcpyAsync(L(c).d_chunks, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    L(c).nchunks = (int)chunks.size();
    L(c).chunk_nt = nt;
    if ((int)strips.size() > L(c).strips_cap) {
        cudaFree(L(c).d_strips);
        L(c).d_strips = nullptr;
        CK(dalloc(&L(c).d_strips, strips.size()));
        L(c).strips_cap = (int)strips.size();
    }
    if (!strips.empty())
        CK(cudaMemcpyAsync(L(c).d_strips, strips.data(), strips.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    L(c).nstrips = (int)strips.size();
    L(c).uform = c->uform;
    L(c).nzones = zoff;
    // The stage lists are used one stage at a time, so every layout shares
    // them; they grow here, while a fold is planned (before its capture), and
    // never shrink. The deferred recovery lists at most every zone; the list
    // of zones above the split at most every zone a P array holds (halo rows
    // included).
    if (zoff > c->high_cap) {
        cudaFree(c->d_high);
        c->d_high = nullptr;
        c->high_cap = 0;
        CK(dalloc(&c->d_high, (size_t)zoff));
        c->high_cap = zoff;
    }
    int64_t padded = 0;
    for (const BlockH* b : order) padded += (b->nr + 4) * b->nq;
    if (padded > c->hp_cap) {
        cudaFree(c->d_hp);
        c->d_hp = nullptr;
        c->hp_cap = 0;
        CK(dalloc(&c->d_hp, (size_t)padded));
        c->hp_cap = padded;
    }
    L(c).tma_ok = false;
    if (tma_ok) {
        if (nb > L(c).tmaps_cap) {
            cudaFree(L(c).d_tmaps);
            L(c).d_tmaps = nullptr;
            CK(dalloc(&L(c).d_tmaps, (size_t)nb));
            L(c).tmaps_cap = nb;
        }
        CK(cudaMemcpyAsync(L(c).d_tmaps, maps.data(), nb * sizeof(TmaMaps), cudaMemcpyHostToDevice, c->stream));
        L(c).tma_ok = true;
    }
    if ((int)remaps.size() > L(c).remap_cap) {
        cudaFree(L(c).d_remap);
        L(c).d_remap = nullptr;
        CK(dalloc(&L(c).d_remap, remaps.size()));
        L(c).remap_cap = (int)remaps.size();
    }
    if (!remaps.empty())
        CK(cudaMemcpyAsync(L(c).d_remap, remaps.data(), remaps.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    L(c).nremap = (int)remaps.size();
    for (int end = 0; end < 2 && nb; ++end) {
        const BlockH& e = *order[end ? nb - 1 : 0];
        L(c).P_edge[end] = e.P;
        L(c).nr_edge[end] = (int32_t)e.nr;
        L(c).nq_edge[end] = (int32_t)e.nq;
        L(c).P64_edge[end] = e.P64;
    }
    CK(cudaStreamSynchronize(c->stream));
    L(c).ntiles = (int)tiles.size();
    c->dirty = false;
    return KNC_OK;
}

// Geometry of the two ghost rows next to the mesh at each end.
int update_ghost_geometry(knc_ctx* c) {
    if (c->blocks.empty()) return KNC_OK;
    const int32_t lo = c->blocks.begin()->first - 1, hi = c->blocks.rbegin()->first + 1;
    // each ghost block has its own radial shape and the polar resolution of
    // the live block it borders
    const int64_t nq_lo = c->blocks.begin()->second.nq, nq_hi = c->blocks.rbegin()->second.nq;
    if (lo == L(c).ghost_lo && hi == L(c).ghost_hi && L(c).d_ghost_rc && nq_lo == L(c).ghost_nq[0] &&
        nq_hi == L(c).ghost_nq[1])
        return KNC_OK;
    const int64_t nr_lo = shape_of(c, lo).first, nr_hi = shape_of(c, hi).first;
    knc_ctx::ColTab* ct;
    int r;
    if ((r = get_cols(c, nq_lo, &ct)) || (r = get_cols(c, nq_hi, &ct))) return r;
    const GeomH gl = make_geometry(c->mesh, lo, false, 1.0, nr_lo, nq_lo);
    const GeomH gh = make_geometry(c->mesh, hi, false, 1.0, nr_hi, nq_hi);
    L(c).ghost_rc_h = {gl.rc[nr_lo - 2], gl.rc[nr_lo - 1], gh.rc[0], gh.rc[1]};
    L(c).ghost_dv_h[0].assign(gl.dv.begin() + (nr_lo - 2) * nq_lo, gl.dv.begin() + nr_lo * nq_lo);
    L(c).ghost_dv_h[1].assign(gh.dv.begin(), gh.dv.begin() + 2 * nq_hi);
    if (!L(c).d_ghost_rc) CK(dalloc(&L(c).d_ghost_rc, 4));
    for (int end = 0; end < 2; ++end) {
        const int64_t nq = end ? nq_hi : nq_lo;
        if (nq != L(c).ghost_nq[end]) {
            cudaFree(L(c).d_ghost_dv[end]);
            L(c).d_ghost_dv[end] = nullptr;
            CK(dalloc(&L(c).d_ghost_dv[end], (size_t)(2 * nq)));
            L(c).ghost_nq[end] = nq;
        }
        CK(cudaMemcpyAsync(L(c).d_ghost_dv[end], L(c).ghost_dv_h[end].data(), 2 * nq * 8, cudaMemcpyHostToDevice,
                           c->stream));
    }
    CK(cudaMemcpyAsync(L(c).d_ghost_rc, L(c).ghost_rc_h.data(), 4 * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    L(c).ghost_lo = lo;
    L(c).ghost_hi = hi;
    return KNC_OK;
}

int ensure_host_prim(knc_ctx* c, size_t n) {
    if (n <= c->host_prim_cap) return KNC_OK;
    cudaFree(c->d_host_prim);
    c->d_host_prim = nullptr;
    CK(dalloc(&c->d_host_prim, n));
    c->host_prim_cap = n;
    return KNC_OK;
}

// Host model values of the ghost rows (slow path: the model is a callback).
int host_ghost_values(knc_ctx* c, double t) {
    const int64_t nq0 = L(c).ghost_nq[0], nq1 = L(c).ghost_nq[1];
    std::vector<double> v((2 * nq0 + 2 * nq1) * 5);
    for (int k = 0; k < 4; ++k) {
        const int end = k / 2;
        const int64_t nq = end ? nq1 : nq0;
        const std::vector<double>& qc = c->cols.at(nq).qc_h;
        const int64_t base = end ? 2 * nq0 : 0;
        for (int64_t j = 0; j < nq; ++j) {
            double any[4], s = 0.0;
            c->host_fn(L(c).ghost_rc_h[k], qc[j], t, any, &s, c->host_user);
            double* o = &v[(base + (int64_t)(k % 2) * nq + j) * 5];
            o[0] = any[2];   // interpret: AnyPrimitive [u_r, u_q, rho, p] -> (rho, u_r, u_q, p)
            o[1] = any[0];
            o[2] = any[1];
            o[3] = any[3];
            o[4] = s;
        }
    }
    int r = ensure_host_prim(c, v.size());
    if (r) return r;
    CK(cudaMemcpyAsync(c->d_host_prim, v.data(), v.size() * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

cudaEvent_t take_event(knc_ctx* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Brackets one launch with events when profiling (not inside graph capture).
struct ProfScope {
    knc_ctx* c;
    int kind;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ProfScope(knc_ctx* c_, int kind_) : c(c_), kind(kind_) {
        if (c->profiling && !c->capturing) {
            e0 = take_event(c);
            e1 = take_event(c);
            cudaEventRecord(e0, c->stream);
        }
    }
    ~ProfScope() {
        if (e0) {
            cudaEventRecord(e1, c->stream);
            c->prof_events.push_back({kind, {e0, e1}});
        }
    }
};

// Fold finished event pairs into the per-kind sums (synchronises on them).
void drain_profile(knc_ctx* c) {
    for (auto& pe : c->prof_events) {
        cudaEventSynchronize(pe.second.second);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
        c->prof_ms[pe.first] += ms;
        c->prof_count[pe.first] += 1;
        c->event_pool.push_back(pe.second.first);
        c->event_pool.push_back(pe.second.second);
    }
    c->prof_events.clear();
}

StageArgs base_args(knc_ctx* c) {
    StageArgs a;
    std::memset(&a, 0, sizeof(a));
    a.blocks = L(c).d_table;
    a.tiles = L(c).d_tiles;
    a.ntiles = L(c).ntiles;
    a.utiles = L(c).d_utiles;
    a.nutiles = L(c).nutiles;
    a.utr = L(c).utr;
    a.tma = c->uform == KNC_UPDATE_TILE_TMA && L(c).tma_ok ? 1 : 0;
    a.tmaps = L(c).tma_ok ? L(c).d_tmaps : nullptr;
    a.strips = c->uform == KNC_UPDATE_STRIP ? L(c).d_strips : nullptr;
    a.nstrips = c->uform == KNC_UPDATE_STRIP ? L(c).nstrips : 0;
    a.strip_ctas = c->ctas_per_sm >= 4 && c->ctas_per_sm <= 6 ? c->ctas_per_sm : 4;
    a.fused_wide = c->fused && c->ctas_per_sm == 1 ? 1 : 0;
    a.srhd = c->hp.system == KNC_SYSTEM_RELATIVISTIC;
    a.hllc = c->hp.riemann_solver == KNC_RIEMANN_HLLC;
    a.one_dimensional = c->mesh.p.num_polar_zones == 1;
    a.guess = c->guess;
    a.gm = c->hp.gamma_law_index;
    a.plm_theta = c->hp.plm_theta;
    a.cflux = a.srhd ? LIGHT_SPEED_H : 1.0;
    a.w_split = c->w_split;
    a.gh = a.gm / (a.gm - 1.0);
    a.gm_f = (float)a.gm;
    a.gm1_f = (float)(a.gm - 1.0);
    a.gh_f = (float)a.gh;
    a.theta_f = (float)a.plm_theta;
    a.cflux_f = (float)a.cflux;
    a.high_thr_f = (float)(1.0 - 1.0 / (c->w_split * c->w_split));
    a.uu_high_f = (float)(c->w_split * c->w_split - 1.0);
    const int le = length_exponent(c->mesh.p);
    a.lscale2 = 2 * le;
    a.lscale3 = 3 * le;
    a.lscale3_d = std::ldexp(1.0, -3 * le);
    a.mlp = c->guess == KNC_GUESS_MLP ? c->d_mlp : nullptr;
    a.status = c->d_status;
    a.sel_base = -1;
    return a;
}

bool mixed(const knc_ctx* c) { return c->precision == KNC_PRECISION_MIXED; }

int launch_c2p(knc_ctx* c, const StageArgs& a) {
    ProfScope ps(c, KNC_KERNEL_C2P);
    cudaError_t e = mixed(c) ? launch_c2p_mixed(a, c->stream) : launch_c2p_f64(a, c->stream);
    // the deferring form is two kernels: every zone, then the deferred ones
    c->launches += mixed(c) && a.high && a.ntiles > 0 ? 2 : 1;
    CK(e);
    return KNC_OK;
}

int launch_update(knc_ctx* c, const StageArgs& a) {
    ProfScope ps(c, KNC_KERNEL_UPDATE);
    cudaError_t e = mixed(c) ? launch_update_mixed(a, c->stream) : launch_update_f64(a, c->stream);
    ++c->launches;
    CK(e);
    return KNC_OK;
}

// CTAs of a fused launch: ctas_per_sm (or the occupancy bound) x SMs, no more
// than the largest phase has work items.
int fused_grid(knc_ctx* c) {
    int per_sm = 1;
    const bool mlp = c->guess == KNC_GUESS_MLP && c->d_mlp;
    const bool strip_only = mixed(c) && c->uform == KNC_UPDATE_STRIP;
    const bool deferred = strip_only && c->rform == KNC_RECOVERY_DEFERRED;
    // StageArgs::fused_wide / strip_ctas: the variant of the deferring form
    const int mb = c->ctas_per_sm == 1 ? 1 : c->ctas_per_sm >= 4 && c->ctas_per_sm <= 6 ? c->ctas_per_sm : 4;
    const cudaError_t e = deferred     ? fused_deferred_max_ctas_mixed(mlp, mb, &per_sm)
                          : strip_only ? fused_strip_max_ctas_mixed(mlp, &per_sm)
                          : mixed(c) ? fused_max_ctas_mixed(mlp, c->utr, &per_sm)
                                     : fused_max_ctas_f64(mlp && c->hp.system == KNC_SYSTEM_RELATIVISTIC, c->utr, &per_sm);
    if (e != cudaSuccess || per_sm < 1) per_sm = 1;
    if (c->ctas_per_sm > 0 && c->ctas_per_sm < per_sm) per_sm = c->ctas_per_sm;
    const Layout& l = L(c);
    const int nt = deferred ? fused_deferred_threads(mb) : fused_threads(c);
    const int need_a = (int)(2 * l.nq_edge[0] + nt - 1) / nt + (int)(2 * l.nq_edge[1] + nt - 1) / nt +
                       (deferred ? (l.ntiles + nt / 32 - 1) / (nt / 32) : l.nchunks);
    const int need_b = (int)(((int64_t)l.nremap * 2 * l.max_nq + nt - 1) / nt);
    const int need_c = l.uform == KNC_UPDATE_STRIP ? (l.nstrips + nt / 32 - 1) / (nt / 32) : l.nutiles;
    const int need = std::max(std::max(need_a, need_b), std::max(need_c, 1));
    return std::min(per_sm * c->sms, need);
}

// One Euler stage U_out = avg(U_in + dt L(U_in), U_base), src/scheme.rs:16-173.
// The arguments of one RK stage's launches (ghost rows, recovery, remaps,
// update); takes the next stage number.
int prepare_stage(knc_ctx* c, int sel_in, int sel_out, int sel_base, double w1, double bf, double t_stage,
                  double dt, int sub, GhostArgs& g, StageArgs& a) {
    int r;
    if (c->stage_counter >= 0xffff) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "too many stages in one call");
    const int32_t stage = c->stage_counter++;
    // ghost rows at the stage time
    std::memset(&g, 0, sizeof(g));
    const Layout& lay = L(c);
    for (int end = 0; end < 2; ++end) {
        g.P[end] = lay.P_edge[end];
        g.nr_t[end] = lay.nr_edge[end];
        g.nq[end] = lay.nq_edge[end];
        g.dv[end] = lay.d_ghost_dv[end];
        g.qc[end] = c->cols.at(lay.nq_edge[end]).qc;
    }
    g.row0[0] = 0;
    g.row0[1] = lay.nr_edge[1] + 2;
    g.ghost_index[0] = lay.ghost_lo;
    g.ghost_index[1] = lay.ghost_hi;
    g.rc = lay.d_ghost_rc;
    g.model = c->model;
    g.time = t_stage;
    g.srhd = c->hp.system == KNC_SYSTEM_RELATIVISTIC;
    g.stage = stage;
    g.gm = c->hp.gamma_law_index;
    g.single_precision = mixed(c) ? 1 : 0;
    if (mixed(c))
        for (int end = 0; end < 2; ++end) g.P64[end] = lay.P_edge[end] ? lay.P64_edge[end] : nullptr;
    g.status = c->d_status;
    if (c->ddt) {
        g.dt_bits = &c->d_status->dt_bits;
        g.cfl = c->hp.cfl_number;
        g.t0 = c->ddt_t0;
        g.order = c->hp.runge_kutta_order;
        g.step = c->ddt_step;
        g.sub = sub;
    }
    if (c->model.kind == KNC_MODEL_HOST) {
        if ((r = host_ghost_values(c, t_stage))) return r;
        g.host_prim[0] = c->d_host_prim;
        g.host_prim[1] = c->d_host_prim + 2 * L(c).ghost_nq[0] * 5;
    }
    a = base_args(c);
    a.stage = stage;
    a.sel_in = sel_in;
    a.sel_out = sel_out;
    a.sel_base = sel_base;
    a.w1 = w1;
    a.bf = bf;
    a.dt = dt;
    a.dt_f = (float)dt;
    a.avg_half = w1 == 0.5 && bf == 0.5 ? 1 : 0;
    if (mixed(c) && c->d_hp) {
        // the list of stored zones above the Lorentz-factor split (written by
        // this stage's recovery, ghost and remap launches, read by its update)
        a.hp_list = c->d_hp;
        a.hp_count = &c->d_status->hp_count[stage & 1];
        a.hp_claim = &c->d_status->hp_claim[stage & 1];
        a.hp_count_next = &c->d_status->hp_count[(stage + 1) & 1];
        a.hp_claim_next = &c->d_status->hp_claim[(stage + 1) & 1];
        a.hp_cap = (unsigned)c->hp_cap;
        g.hp_list = a.hp_list;
        g.hp_count = a.hp_count;
        g.hp_cap = a.hp_cap;
        g.edge_slot[0] = 0;
        g.edge_slot[1] = (int32_t)L(c).slot_index.size() - 1;
        g.uu_high_f = a.uu_high_f;
    }
    if (mixed(c) && (!c->fused || c->uform == KNC_UPDATE_STRIP) && c->rform == KNC_RECOVERY_DEFERRED && c->d_high) {
        a.high = c->d_high;
        a.high_count = &c->d_status->high_count[stage & 1];
        a.high_count_next = &c->d_status->high_count[(stage + 1) & 1];
        a.high_cap = (unsigned)c->high_cap;
    }
    if (c->ddt) {
        a.dt_bits = &c->d_status->dt_bits;
        a.cfl = c->hp.cfl_number;
        a.compute_dt = c->ddt_step == 0 && sub == 0 ? 1 : 0;   // the fold's first recovery finds dt
    }
    return KNC_OK;
}

int run_stage(knc_ctx* c, int sel_in, int sel_out, int sel_base, double w1, double bf, double t_stage,
              double dt, int sub) {
    int r;
    GhostArgs g;
    StageArgs a;
    if ((r = prepare_stage(c, sel_in, sel_out, sel_base, w1, bf, t_stage, dt, sub, g, a))) return r;
    const Layout& lay = L(c);
    if (c->fused) {
        // the whole stage in one cooperative launch (grid barriers between phases)
        FusedArgs f;
        std::memset(&f, 0, sizeof(f));
        f.chunks = lay.d_chunks;
        f.nchunks = lay.nchunks;
        f.nremap = lay.nremap;
        f.remap = lay.d_remap;
        f.max_nq = lay.max_nq;
        // the wait test: a poll limit of its own, and a first barrier that
        // counts one arrival more than the grid makes (it cannot complete)
        f.spin_limit = c->wait_polls > 0 ? c->wait_polls : BARRIER_SPIN_LIMIT;
        f.bar_base = c->bar_epoch + (c->wait_unreachable ? 1u : 0u);
        const int grid = fused_grid(c);
        // barrier arrivals per CTA: the deferring form always counts three
        const bool deferred = mixed(c) && c->uform == KNC_UPDATE_STRIP && c->rform == KNC_RECOVERY_DEFERRED;
        c->bar_epoch += (unsigned long long)grid * (deferred ? 3u : lay.nremap ? 2u : 1u);
        ProfScope ps(c, KNC_KERNEL_FUSED);
        CK(mixed(c) ? launch_stage_fused_mixed(a, g, f, grid, c->stream)
                    : launch_stage_fused_f64(a, g, f, grid, c->stream));
        ++c->launches;
        return KNC_OK;
    }
    if (c->profiling) {
        // timed one kernel after another
        {
            ProfScope ps(c, KNC_KERNEL_GHOST);
            CK(mixed(c) ? launch_ghost_mixed(g, c->stream) : launch_ghost_f64(g, c->stream));
        }
        if ((r = launch_c2p(c, a))) return r;
    } else {
        // the ghost rows (mesh-end halos, a short FP64 latency chain) beside the
        // recovery, which writes interior rows and inner halos only
        CK(cudaEventRecord(c->ev_fork, c->stream));
        CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        CK(mixed(c) ? launch_ghost_mixed(g, c->side) : launch_ghost_f64(g, c->side));
        CK(cudaEventRecord(c->ev_join, c->side));
        if ((r = launch_c2p(c, a))) return r;
        CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    }
    ++c->launches;
    if (lay.nremap) {
        CK(mixed(c) ? launch_remap_mixed(a, lay.d_remap, lay.nremap, lay.max_nq, c->stream)
                    : launch_remap_f64(a, lay.d_remap, lay.nremap, lay.max_nq, c->stream));
        ++c->launches;
    }
    if ((r = launch_update(c, a))) return r;
    return KNC_OK;
}

// Stage start times of one SSP RK step and the time after it, averaged as
// godunov_core::runge_kutta does (t = t1 (1 - b) + t0 b). rk_step and the
// planner of a captured fold both take their times from here.
struct StepTimes {
    double stage[3];
    double end;
};

StepTimes step_times(int order, double t0, double dt) {
    auto avg_time = [](double t1, double tb, double bf) { return t1 * (-bf + 1.0) + tb * bf; };
    StepTimes s{};
    s.stage[0] = t0;
    const double t1 = t0 + dt;
    if (order == 1) {
        s.end = t1;
        return s;
    }
    s.stage[1] = t1;
    if (order == 2) {
        s.end = avg_time(t1 + dt, t0, 0.5);
        return s;
    }
    const double t2 = avg_time(t1 + dt, t0, 0.75);
    s.stage[2] = t2;
    s.end = avg_time(t2 + dt, t0, 1.0 / 3.0);
    return s;
}

// The stages of one SSP RK step (godunov_core::runge_kutta::try_advance_async
// restated, RK1/RK2/RK3): the input, output and base buffers of each stage,
// its averaging weights (1 - b) and b, and its start time.
struct StagePlan {
    int sel_in, sel_out, sel_base;
    double w1, bf, t;
    int sub;
};

int step_plan(const knc_ctx* c, double dt, StagePlan p[3]) {
    const int A = c->cur, B = 1 - c->cur;
    const int order = c->hp.runge_kutta_order;
    const StepTimes T = step_times(order, c->time, dt);
    p[0] = {A, B, -1, 1.0, 0.0, T.stage[0], 0};
    if (order == 1) return 1;
    if (order == 2) {
        const double bf = 0.5;
        p[1] = {B, A, A, -bf + 1.0, bf, T.stage[1], 1};
        return 2;
    }
    const double b2 = 0.75, b3 = 1.0 / 3.0;
    p[1] = {B, B, A, -b2 + 1.0, b2, T.stage[1], 1};
    p[2] = {B, A, A, -b3 + 1.0, b3, T.stage[2], 2};
    return 3;
}

// Time, iteration and current buffer after a step's stages ran.
void finish_step(knc_ctx* c, double dt) {
    const double t0 = c->time;
    const Rational it0 = c->iteration;
    Rational one;
    one.n = 1;
    const int order = c->hp.runge_kutta_order;
    const StepTimes T = step_times(order, t0, dt);
    auto avg_iter = [&](Rational i1, Rational br) {
        Rational mbr = br;
        mbr.n = -mbr.n;
        return i1.mul(mbr.add(one)).add(it0.mul(br));
    };
    const Rational i1 = it0.add(one);
    if (!c->ddt) c->time = T.end;
    if (order == 1) {
        c->cur = 1 - c->cur;
        c->iteration = i1;
    } else if (order == 2) {
        Rational half;
        half.n = 1;
        half.d = 2;
        c->iteration = avg_iter(i1.add(one), half);
    } else {
        Rational q34, q13;
        q34.n = 3;
        q34.d = 4;
        q13.n = 1;
        q13.d = 3;
        const Rational i2 = avg_iter(i1.add(one), q34);
        c->iteration = avg_iter(i2.add(one), q13);
    }
}

int rk_step(knc_ctx* c, double dt) {
    StagePlan p[3];
    const int n = step_plan(c, dt, p);
    c->zone_updates += L(c).nzones;
    int r;
    for (int s = 0; s < n; ++s)
        if ((r = run_stage(c, p[s].sel_in, p[s].sel_out, p[s].sel_base, p[s].w1, p[s].bf, p[s].t, dt, p[s].sub)))
            return r;
    finish_step(c, dt);
    return KNC_OK;
}

// Read the device status; on a hydro failure fill c->err from the failing zone.
int check_status(knc_ctx* c) {
    CK(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const unsigned long long k = c->h_status->err_key;
    if (c->h_status->bar_abort) {
        c->failed = true;
        return set_msg(c, KNC_ERR_TIMEOUT, "a grid barrier of the fused stage timed out");
    }
    if (k == NO_ERROR) return KNC_OK;
    c->failed = true;
    const uint32_t slot = (uint32_t)((k >> 34) & 0x3fffu);
    const int32_t i = (int32_t)((k >> 20) & 0x3fffu);
    const int32_t j = (int32_t)((k >> 4) & 0xffffu);
    const int32_t kind = (int32_t)(k & 0xfu);
    const int32_t stage = (int32_t)(k >> 48);
    std::memset(&c->err, 0, sizeof(c->err));
    c->err.kind = kind;
    c->err.i = i;
    c->err.j = j;
    // the layout in effect at the failing stage (layouts are in stage order)
    const Layout* lay = &c->lays.front();
    for (const Layout& l : c->lays)
        if (l.first_stage <= stage) lay = &l;
    if (slot >= 0x3ffeu) {
        const int end = (int)(slot - 0x3ffeu);
        c->err.block = end ? lay->ghost_hi : lay->ghost_lo;
        c->err.r = lay->ghost_rc_h.empty() ? 0.0 : lay->ghost_rc_h[end * 2 + i];
        auto ct = c->cols.find(lay->ghost_nq[end]);
        c->err.theta = ct == c->cols.end() ? 0.0 : ct->second.qc_h[j];
    } else if (slot < lay->slot_index.size()) {
        const int32_t index = lay->slot_index[slot];
        c->err.block = index;
        const BlockH* bp = nullptr;
        auto it = c->blocks.find(index);
        if (it != c->blocks.end()) bp = &it->second;
        for (const BlockH& d : c->deferred)
            if (d.index == index) bp = &d;
        if (bp) {
            const BlockH& b = *bp;
            c->err.r = b.geom.rc[i];
            c->err.theta = c->cols.at(b.nq).qc_h[j];
            const int sel = c->h_status->err_sel;
            double u[5];
            const int64_t n = b.nr * b.nq, z = (int64_t)i * b.nq + j;
            for (int q = 0; q < 5; ++q)
                CK(cudaMemcpy(&u[q], b.buf[sel] + q * n + z, 8, cudaMemcpyDeviceToHost));
            const double dV = b.geom.dv[z];
            c->err.value = kind == KNC_HYDRO_NEGATIVE_ENERGY_DENSITY ? u[3] / dV : u[0] / dV;
        }
    }
    static const char* names[] = {"None", "NegativeDensity", "NegativePressure", "NegativeEnergyDensity",
                                  "RootFinderFailed"};
    std::snprintf(c->err.message, sizeof(c->err.message),
                  "%s(%.4e) at position (r, theta) = (%.4e, %.4f) in block %d zone (%d, %d)",
                  names[kind <= 4 ? kind : 0], c->err.value, c->err.r, c->err.theta, c->err.block, i, j);
    return KNC_ERR_HYDRO;
}

int reset_status(knc_ctx* c, bool keep_stats) {
    DevStatus* d = c->d_status;
    if (keep_stats) {
        // stream-ordered field writes, no round trip: the error key and dt
        // minimum to all-ones, the barrier and deferral counters to zero
        CK(cudaMemsetAsync(&d->err_key, 0xff, sizeof(d->err_key), c->stream));
        CK(cudaMemsetAsync(&d->err_sel, 0, sizeof(d->err_sel), c->stream));
        CK(cudaMemsetAsync(&d->dt_bits, 0xff, sizeof(d->dt_bits), c->stream));
        CK(cudaMemsetAsync(&d->bar_count, 0, sizeof(d->bar_count) + sizeof(d->bar_abort), c->stream));
        CK(cudaMemsetAsync(d->high_count, 0, sizeof(d->high_count), c->stream));
        CK(cudaMemsetAsync(d->hp_count, 0, sizeof(d->hp_count) + sizeof(d->hp_claim), c->stream));
        // the fused deferring stage's item counter: a launch whose grid
        // barrier gave up may leave it counting
        CK(cudaMemsetAsync(&d->item_claim, 0, sizeof(d->item_claim), c->stream));
    } else {
        DevStatus s;
        std::memset(&s, 0, sizeof(s));
        s.err_key = NO_ERROR;
        s.dt_bits = ~0ull;
        CK(cudaMemcpyAsync(d, &s, sizeof(s), cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    c->bar_epoch = 0;
    c->stage_counter = 0;
    return KNC_OK;
}

int init_block_from_model(knc_ctx* c, int32_t index, double t) {
    // the new block is the last slot; run the init kernel on its tiles only
    int r;
    if ((r = rebuild_table(c))) return r;
    int slot = -1;
    for (size_t k = 0; k < L(c).slot_index.size(); ++k)
        if (L(c).slot_index[k] == index) slot = (int)k;
    if (slot < 0) return set_msg(c, KNC_ERR_NO_BLOCK, "block %d missing", index);
    std::vector<int4> tiles;
    const BlockH& b = c->blocks.at(index);
    for (int64_t i0 = 0; i0 < b.nr; i0 += TILE_R)
        for (int64_t j0 = 0; j0 < b.nq; j0 += TILE_Q) tiles.push_back(make_int4(slot, (int)i0, (int)j0, 0));
    int4* d_t = nullptr;
    CK(dalloc(&d_t, tiles.size()));
    CK(cudaMemcpyAsync(d_t, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
    InitArgs ia;
    std::memset(&ia, 0, sizeof(ia));
    ia.blocks = L(c).d_table;
    ia.tiles = d_t;
    ia.sel = c->cur;
    ia.srhd = c->hp.system == KNC_SYSTEM_RELATIVISTIC;
    ia.noise = 0;   // activated blocks take the model's noise-free data, like ghosts
    ia.gm = c->hp.gamma_law_index;
    ia.time = t;
    ia.model = c->model;
    if (c->model.kind == KNC_MODEL_HOST) {
        const int64_t nz = b.nr * b.nq;
        std::vector<double> v(nz * 5);
        for (int64_t i = 0; i < b.nr; ++i)
            for (int64_t j = 0; j < b.nq; ++j) {
                double any[4], s = 0.0;
                c->host_fn(b.geom.rc[i], b.geom.qc[j], t, any, &s, c->host_user);
                double* o = &v[(i * b.nq + j) * 5];
                o[0] = any[2];
                o[1] = any[0];
                o[2] = any[1];
                o[3] = any[3];
                o[4] = s;
            }
        if ((r = ensure_host_prim(c, v.size()))) return r;
        CK(cudaMemcpyAsync(c->d_host_prim, v.data(), v.size() * 8, cudaMemcpyHostToDevice, c->stream));
        ia.host_prim = c->d_host_prim;
    }
    cudaError_t e = launch_init_f64(ia, (int)tiles.size(), c->stream);
    ++c->launches;
    cudaError_t e2 = cudaStreamSynchronize(c->stream);
    cudaFree(d_t);
    CK(e);
    CK(e2);
    return KNC_OK;
}

int insert_block(knc_ctx* c, int32_t index) {
    auto it = c->blocks.find(index);
    if (it != c->blocks.end()) return KNC_OK;
    BlockH b;
    int r = alloc_block(c, index, b);
    if (r) return r;
    c->blocks.emplace(index, b);
    c->dirty = true;
    return KNC_OK;
}

// add_remove_blocks, src/scheme.rs:179-206
int add_remove_blocks(knc_ctx* c) {
    if (c->blocks.empty()) return KNC_OK;
    const int32_t inner = c->blocks.begin()->first;
    const int32_t outer = c->blocks.rbegin()->first;
    const bool drop = c->mesh.extent(inner).r1 < c->mesh.ies(c->time);
    const bool add = c->mesh.extent(outer).r1 < c->mesh.oes(c->time);
    if (!drop && !add) return KNC_OK;
    int r;
    // surface errors of the steps so far before the slot layout changes
    if ((r = check_status(c))) return r;
    if (drop) {
        release_block(c, c->blocks.at(inner));
        c->blocks.erase(inner);
        c->dirty = true;
    }
    if (add) {
        const int32_t nb = outer + 1;
        if ((r = insert_block(c, nb))) return r;
        if ((r = init_block_from_model(c, nb, c->time))) return r;
        // initial data of an activated block is noise-free, as for ghosts
    }
    if ((r = rebuild_table(c))) return r;
    if ((r = update_ghost_geometry(c))) return r;
    return KNC_OK;
}

int check_ready(knc_ctx* c) {
    if (c->blocks.empty()) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "no blocks");
    if (!c->have_model) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "no model set (ghost blocks need one)");
    int32_t prev = INT32_MIN;
    for (auto& kv : c->blocks) {
        if (prev != INT32_MIN && kv.first != prev + 1)
            return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "block indexes are not contiguous (%d after %d)",
                           kv.first, prev);
        prev = kv.first;
    }
    if (c->failed) return set_msg(c, KNC_ERR_HYDRO, "state invalid after an earlier hydro error: %s",
                                  c->err.message);
    if (mixed(c) && c->hp.system != KNC_SYSTEM_RELATIVISTIC)
        return set_msg(c, KNC_ERR_UNSUPPORTED, "the mixed-precision stage is built for relativistic hydro");
    if (c->mesh.p.num_polar_zones == 1 && mixed(c))
        return set_msg(c, KNC_ERR_UNSUPPORTED, "mixed precision needs num_polar_zones > 1");
    return KNC_OK;
}

int time_step_impl(knc_ctx* c, double* dt) {
    const bool global = c->hp.system == KNC_SYSTEM_RELATIVISTIC && !c->hp.adaptive_time_step;
    if (global) {   // cfl * smallest_spacing(innermost) / c, state.rs:147-149
        // With uneven blocks a finer block further out can hold the smallest
        // spacing, so the minimum runs over all blocks; for equal shapes the
        // innermost block is always the minimum and this is the reference rule.
        double spacing = 0.0;
        bool have = false;
        for (auto& kv : c->blocks) {
            const ExtentH e = c->mesh.extent(kv.first);
            const int64_t nr = kv.second.nr;
            const double sp = vertex_r(e, nr, 1) - vertex_r(e, nr, 0);
            if (!have || sp < spacing) spacing = sp;
            have = true;
        }
        *dt = c->hp.cfl_number * spacing / LIGHT_SPEED_H;
        return KNC_OK;
    }
    int r;
    if ((r = rebuild_table(c))) return r;
    // adaptive: full c2p pass with the dl / a_max reduction
    unsigned long long big = ~0ull;
    CK(cudaMemcpyAsync(&c->d_status->dt_bits, &big, 8, cudaMemcpyHostToDevice, c->stream));
    StageArgs a = base_args(c);
    a.stage = c->stage_counter++;
    a.sel_in = c->cur;
    a.sel_out = c->cur;
    a.compute_dt = 1;
    // the reduction runs in the FP64 c2p kernel whatever the precision mode
    CK(launch_c2p_f64(a, c->stream));
    ++c->launches;
    if ((r = check_status(c))) return r;
    double dtmin;
    std::memcpy(&dtmin, &c->h_status->dt_bits, 8);
    *dt = dtmin * c->hp.cfl_number;
    return KNC_OK;
}

int ensure_stage(knc_ctx* c, size_t doubles) {
    if (doubles <= c->stage_cap) return KNC_OK;
    cudaFree(c->d_stage);
    c->d_stage = nullptr;
    CK(dalloc(&c->d_stage, doubles));
    c->stage_cap = doubles;
    return KNC_OK;
}

int create_device_side(knc_ctx* c) {
    int r;
    CK(configure_kernels());
    CK(cudaGetDevice(&c->device));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->h2d, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->d2h, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    {
        int coop = 0;
        CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
        CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
        c->coop = coop != 0;
    }
    CK(dalloc(&c->d_status, 1));
    CK(cudaMallocHost((void**)&c->h_status, sizeof(DevStatus)));
    knc_ctx::ColTab* ct;
    if ((r = get_cols(c, c->mesh.p.num_polar_zones, &ct))) return r;
    return reset_status(c, false);
}

}  // namespace

namespace knc {
void host_block_volumes(const knc_mesh_params& mesh, int32_t index, std::vector<double>& dv,
                        std::vector<double>& rc, std::vector<double>& qc) {
    MeshH M;
    M.p = mesh;
    GeomH G = make_geometry(M, index, false);
    dv.swap(G.dv);
    rc.swap(G.rc);
    qc.swap(G.qc);
}
}  // namespace knc

// =========================================================================== C ABI
extern "C" {

const char* knc_status_string(int s) {
    switch (s) {
    case KNC_OK: return "ok";
    case KNC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KNC_ERR_CONFIG: return "invalid configuration";
    case KNC_ERR_CUDA: return "CUDA error";
    case KNC_ERR_NO_BLOCK: return "no such block";
    case KNC_ERR_HYDRO: return "hydro error";
    case KNC_ERR_UNSUPPORTED: return "unsupported";
    case KNC_ERR_OUT_OF_MEMORY: return "out of device memory";
    case KNC_ERR_TIMEOUT: return "timeout";
    default: return "unknown status";
    }
}

int knc_create(const knc_hydro_params* hydro, const knc_mesh_params* mesh, knc_ctx** out) {
    if (!hydro || !mesh || !out) return KNC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    knc_ctx* c = new knc_ctx();
    int r = validate(c, hydro, mesh);
    if (r) { delete c; return r; }
    c->hp = *hydro;
    c->mesh.p = *mesh;
    c->iteration.n = 0;
    c->iteration.d = 1;
    r = create_device_side(c);
    if (r) { knc_destroy(c); return r; }
    *out = c;
    return KNC_OK;
}

void knc_destroy(knc_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& kv : c->blocks) free_block(kv.second);
    for (auto& kv : c->pool)
        for (auto& b : kv.second) free_block(b);
    for (auto& kv : c->cols) {
        knc_ctx::ColTab& t = kv.second;
        cudaFree(t.qv);
        cudaFree(t.qc);
        cudaFree(t.cot);
        cudaFree(t.ar_q);
        cudaFree(t.aq_q);
        cudaFree(t.dv_q);
        cudaFree(t.cot32);
    }
    for (auto& l : c->lays) free_layout(l);
    for (auto& b : c->deferred) free_block(b);
    cudaFree(c->d_host_prim);
    cudaFree(c->d_status);
    cudaFree(c->d_mlp);
    cudaFree(c->d_high);
    cudaFree(c->d_hp);
    cudaFree(c->d_stage);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    for (cudaEvent_t e : c->marks)
        if (e) cudaEventDestroy(e);
    drain_profile(c);
    for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    for (cudaStream_t st : {c->h2d, c->d2h})
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (cudaStream_t st : c->kstreams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    for (cudaEvent_t e : c->ev_chunk) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int knc_last_error(const knc_ctx* c, knc_error* out) {
    if (!c || !out) return KNC_ERR_INVALID_ARGUMENT;
    *out = c->err;
    return KNC_OK;
}

int knc_set_model(knc_ctx* c, const knc_model_params* m) {
    if (!c || !m) return KNC_ERR_INVALID_ARGUMENT;
    if (m->kind < KNC_MODEL_WIND || m->kind > KNC_MODEL_JET_IN_STAR || m->kind == KNC_MODEL_HOST)
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "unknown model kind %d", m->kind);
    c->model = *m;
    c->have_model = true;
    return KNC_OK;
}

int knc_set_host_model(knc_ctx* c, knc_primitive_at_fn fn, void* user) {
    if (!c || !fn) return KNC_ERR_INVALID_ARGUMENT;
    std::memset(&c->model, 0, sizeof(c->model));
    c->model.kind = KNC_MODEL_HOST;
    c->host_fn = fn;
    c->host_user = user;
    c->have_model = true;
    return KNC_OK;
}

int knc_init_from_model(knc_ctx* c, double time) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (!c->have_model) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "no model set");
    if (c->mesh.p.reference_radius > c->mesh.oes(time))
        return set_msg(c, KNC_ERR_CONFIG, "the reference radius is outside the outer excision surface");
    int r;
    CK(cudaStreamSynchronize(c->stream));
    for (auto& kv : c->blocks) release_block(c, kv.second);
    c->blocks.clear();
    c->dirty = true;
    std::vector<int32_t> idx;
    for (int32_t i = 0;; ++i) {                              // Mesh::grid_blocks, mesh.rs:384-397
        if (c->mesh.extent(i).r0 >= c->mesh.oes(time)) break;
        idx.push_back(i);
        if (i > 100000) return set_msg(c, KNC_ERR_CONFIG, "mesh has more than 100000 blocks");
    }
    c->cur = 0;
    for (int32_t i : idx)
        if ((r = insert_block(c, i))) return r;
    if ((r = rebuild_table(c))) return r;
    InitArgs ia;
    std::memset(&ia, 0, sizeof(ia));
    ia.blocks = L(c).d_table;
    ia.tiles = L(c).d_tiles;
    ia.sel = c->cur;
    ia.srhd = c->hp.system == KNC_SYSTEM_RELATIVISTIC;
    ia.noise = 1;
    ia.gm = c->hp.gamma_law_index;
    ia.time = time;
    ia.model = c->model;
    if (c->model.kind == KNC_MODEL_HOST) {
        int64_t nz = 0;
        for (auto& kv : c->blocks) nz += kv.second.nr * kv.second.nq;
        std::vector<double> v(nz * 5);
        int64_t off = 0;
        for (auto& kv : c->blocks) {
            const BlockH& b = kv.second;
            for (int64_t i = 0; i < b.nr; ++i)
                for (int64_t j = 0; j < b.nq; ++j) {
                    double any[4], s = 0.0;
                    c->host_fn(b.geom.rc[i], b.geom.qc[j], time, any, &s, c->host_user);
                    double* o = &v[(off + i * b.nq + j) * 5];
                    o[0] = any[2];
                    o[1] = any[0];
                    o[2] = any[1];
                    o[3] = any[3];
                    o[4] = s;
                }
            off += b.nr * b.nq;
        }
        if ((r = ensure_host_prim(c, v.size()))) return r;
        CK(cudaMemcpyAsync(c->d_host_prim, v.data(), v.size() * 8, cudaMemcpyHostToDevice, c->stream));
        ia.host_prim = c->d_host_prim;
    }
    CK(launch_init_f64(ia, L(c).ntiles, c->stream));
    ++c->launches;
    CK(cudaStreamSynchronize(c->stream));
    c->time = time;
    c->iteration.n = 0;
    c->iteration.d = 1;
    c->failed = false;
    if ((r = reset_status(c, true))) return r;
    return update_ghost_geometry(c);
}

int knc_add_block(knc_ctx* c, int32_t index, const double* cons, const double* scalar) {
    if (!c || !cons || !scalar) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = insert_block(c, index))) return r;
    BlockH& b = c->blocks.at(index);
    const size_t n = (size_t)(b.nr * b.nq);
    if ((r = ensure_stage(c, 5 * n))) return r;
    CK(cudaMemcpyAsync(c->d_stage, cons, 4 * n * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_stage + 4 * n, scalar, n * 8, cudaMemcpyHostToDevice, c->stream));
    CK(launch_aos_to_soa(c->d_stage, c->d_stage + 4 * n, b.buf[c->cur], b.nr, b.nq, c->stream));
    ++c->launches;
    CK(cudaStreamSynchronize(c->stream));
    c->failed = false;
    if ((r = reset_status(c, true))) return r;
    return update_ghost_geometry(c);
}

int knc_remove_block(knc_ctx* c, int32_t index) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return set_msg(c, KNC_ERR_NO_BLOCK, "no block %d", index);
    CK(cudaStreamSynchronize(c->stream));
    release_block(c, it->second);
    c->blocks.erase(it);
    c->dirty = true;
    return c->blocks.empty() ? KNC_OK : update_ghost_geometry(c);
}

int knc_get_block(knc_ctx* c, int32_t index, double* cons, double* scalar) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return set_msg(c, KNC_ERR_NO_BLOCK, "no block %d", index);
    const BlockH& b = it->second;
    const size_t n = (size_t)(b.nr * b.nq);
    int r;
    if ((r = ensure_stage(c, 5 * n))) return r;
    CK(launch_soa_to_aos(b.buf[c->cur], c->d_stage, c->d_stage + 4 * n, b.nr, b.nq, c->stream));
    ++c->launches;
    if (cons) CK(cudaMemcpyAsync(cons, c->d_stage, 4 * n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (scalar) CK(cudaMemcpyAsync(scalar, c->d_stage + 4 * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

int knc_num_blocks(const knc_ctx* c, int32_t* n) {
    if (!c || !n) return KNC_ERR_INVALID_ARGUMENT;
    *n = (int32_t)c->blocks.size();
    return KNC_OK;
}

int knc_block_indexes(const knc_ctx* c, int32_t* out, int32_t capacity) {
    if (!c || !out) return KNC_ERR_INVALID_ARGUMENT;
    if ((int32_t)c->blocks.size() > capacity) return KNC_ERR_INVALID_ARGUMENT;
    int32_t k = 0;
    for (auto& kv : c->blocks) out[k++] = kv.first;
    return KNC_OK;
}

int knc_block_shape(const knc_ctx* c, int64_t* nr, int64_t* nq) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (nr) *nr = c->mesh.p.block_size;
    if (nq) *nq = c->mesh.p.num_polar_zones;
    return KNC_OK;
}

int knc_set_block_shapes(knc_ctx* c, int32_t first, int32_t count, const int32_t* nr, const int32_t* nq) {
    if (!c || count < 0 || (count && (!nr || !nq))) return KNC_ERR_INVALID_ARGUMENT;
    const int64_t nq0 = c->mesh.p.num_polar_zones;
    for (int32_t k = 0; k < count; ++k) {
        if (nr[k] < 2 || nr[k] > 16383)
            return set_msg(c, KNC_ERR_CONFIG, "block %d: radial zones %d outside [2, 16383]", first + k, nr[k]);
        bool pow2 = false;   // nq = nq0 * 2^m for some integer m
        for (int64_t a = nq0, b = nq[k]; !pow2 && a > 0 && b > 0;) {
            if (a == b) pow2 = true;
            else if (a < b) { if (b % 2) break; b /= 2; }
            else { if (a % 2) break; a /= 2; }
        }
        if (!pow2 || nq[k] > 65535 || (nq0 != 1 && nq[k] < 16) || (nq0 == 1 && nq[k] != 1))
            return set_msg(c, KNC_ERR_CONFIG,
                           "block %d: polar zones %d must be the mesh's %lld times a power of two, in [16, 65535]",
                           first + k, nq[k], (long long)nq0);
        auto it = c->blocks.find(first + k);
        if (it != c->blocks.end() && (it->second.nr != nr[k] || it->second.nq != nq[k]))
            return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "block %d is live with another shape", first + k);
    }
    for (int32_t k = 0; k < count; ++k) c->shapes[first + k] = {nr[k], nq[k]};
    L(c).ghost_lo = INT32_MIN;   // ghost shapes may have changed
    c->dirty = true;
    return c->blocks.empty() ? KNC_OK : update_ghost_geometry(c);
}

int knc_block_shape_of(const knc_ctx* c, int32_t index, int64_t* nr, int64_t* nq) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    const auto sh = shape_of(c, index);
    if (nr) *nr = sh.first;
    if (nq) *nq = sh.second;
    return KNC_OK;
}

// The device address of host memory the GPU can read and write directly
// (page-locked or registered; over NVLink-C2C on a Grace host), else null.
const void* device_view(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
    return nullptr;
}

int knc_set_state(knc_ctx* c, const double* cons, const double* scalar) {
    if (!c || !cons || !scalar) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = rebuild_table(c))) return r;
    int64_t total = 0;
    for (auto& kv : c->blocks) total += kv.second.nr * kv.second.nq;
    const double* dc = static_cast<const double*>(device_view(cons));
    const double* ds = static_cast<const double*>(device_view(scalar));
    if (!dc || !ds) {
        // pageable host memory: through a device staging copy
        if ((r = ensure_stage(c, 5 * (size_t)total))) return r;
        CK(cudaMemcpyAsync(c->d_stage, cons, 4 * total * 8, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->d_stage + 4 * total, scalar, total * 8, cudaMemcpyHostToDevice, c->stream));
        dc = c->d_stage;
        ds = c->d_stage + 4 * total;
    }
    // one launch reads the arrays (directly from page-locked host memory when
    // it can: on GB300 that beat a DMA copy plus transpose, 0.81 vs 0.87 ms
    // for 168 MB) and writes every block's SoA state
    CK(launch_state_in(L(c).d_table, L(c).d_tiles, L(c).ntiles, c->cur, dc, ds, c->stream));
    ++c->launches;
    // the caller's buffers are free again when the call returns
    CK(cudaStreamSynchronize(c->stream));
    c->failed = false;
    return KNC_OK;
}

int knc_get_state(knc_ctx* c, double* cons, double* scalar) {
    if (!c || !cons || !scalar) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = rebuild_table(c))) return r;
    int64_t total = 0;
    for (auto& kv : c->blocks) total += kv.second.nr * kv.second.nq;
    // transposed on the device, then one DMA copy per array: measured on
    // GB300, writing host memory from a kernel is slower than the copy engines
    if ((r = ensure_stage(c, 5 * (size_t)total))) return r;
    CK(launch_state_out(L(c).d_table, L(c).d_tiles, L(c).ntiles, c->cur, c->d_stage, c->d_stage + 4 * total,
                        c->stream));
    ++c->launches;
    CK(cudaMemcpyAsync(cons, c->d_stage, 4 * total * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(scalar, c->d_stage + 4 * total, total * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

int knc_set_time(knc_ctx* c, double time, int64_t num, int64_t den) {
    if (!c || den == 0) return KNC_ERR_INVALID_ARGUMENT;
    c->time = time;
    c->iteration.n = num;
    c->iteration.d = den;
    c->iteration.norm();
    return KNC_OK;
}

int knc_get_time(const knc_ctx* c, double* time, int64_t* num, int64_t* den) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (time) *time = c->time;
    if (num) *num = c->iteration.n;
    if (den) *den = c->iteration.d;
    return KNC_OK;
}

int knc_time_step(knc_ctx* c, double* dt) {
    if (!c || !dt) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = check_ready(c))) return r;
    if ((r = reset_status(c, true))) return r;
    return time_step_impl(c, dt);
}

namespace {

// Block-set changes of a captured fold whose excision surfaces move, decided
// on the host before capture: the step times come from step_times (the same
// arithmetic rk_step applies), so each step's add_remove_blocks outcome
// (src/scheme.rs:179-206) is known in advance. Every block set gets its own
// layout with fresh device buffers; an activated block is allocated now and
// its initial data is written by an init launch inside the graph at the step
// it joins; a retired block's storage is held until the graph has run.
int plan_fold(knc_ctx* c, int32_t fold, double dt, std::vector<int>& step_lay, std::vector<char>& step_init) {
    double t = c->time;
    const int order = c->hp.runge_kutta_order;
    int r;
    for (int32_t k = 0; k < fold; ++k) {
        const int32_t inner = c->blocks.begin()->first;
        const int32_t outer = c->blocks.rbegin()->first;
        const bool drop = c->mesh.extent(inner).r1 < c->mesh.ies(t);
        const bool add = c->mesh.extent(outer).r1 < c->mesh.oes(t);
        if (drop || add) {
            if (drop) {
                if (c->blocks.size() == 1 && !add)
                    return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "the inner excision surface removed every block");
                c->deferred.push_back(c->blocks.at(inner));
                c->blocks.erase(inner);
            }
            if (add && (r = insert_block(c, outer + 1))) return r;
            c->lays.emplace_back();
            c->cur_lay = (int)c->lays.size() - 1;
            c->dirty = true;
            if ((r = rebuild_table(c))) return r;
            if ((r = update_ghost_geometry(c))) return r;
            if (add) {
                const BlockH& b = c->blocks.at(outer + 1);
                const int slot = (int)L(c).slot_index.size() - 1;   // the outermost slot
                std::vector<int4> tiles;
                for (int64_t i0 = 0; i0 < b.nr; i0 += TILE_R)
                    for (int64_t j0 = 0; j0 < b.nq; j0 += TILE_Q) tiles.push_back(make_int4(slot, (int)i0, (int)j0, 0));
                CK(upload(&L(c).d_init_tiles, tiles, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                L(c).n_init_tiles = (int)tiles.size();
            }
        }
        step_lay[k] = c->cur_lay;
        step_init[k] = add ? 1 : 0;
        t = step_times(order, t, dt).end;
    }
    return KNC_OK;
}

// Initial data of the block activated at the start of this step (captured).
int launch_activation(knc_ctx* c) {
    InitArgs ia;
    std::memset(&ia, 0, sizeof(ia));
    ia.blocks = L(c).d_table;
    ia.tiles = L(c).d_init_tiles;
    ia.sel = c->cur;
    ia.srhd = c->hp.system == KNC_SYSTEM_RELATIVISTIC;
    ia.noise = 0;   // activated blocks take the model's noise-free data, like ghosts
    ia.gm = c->hp.gamma_law_index;
    ia.time = c->time;
    ia.model = c->model;
    CK(launch_init_f64(ia, L(c).n_init_tiles, c->stream));
    ++c->launches;
    return KNC_OK;
}

// After a captured fold ran: keep the last layout, free the others, and
// return retired blocks' storage to the pool.
void finish_fold(knc_ctx* c) {
    if (c->lays.size() > 1) {
        Layout keep = c->lays[c->cur_lay];
        c->lays[c->cur_lay] = Layout();
        for (auto& l : c->lays) free_layout(l);
        c->lays.assign(1, keep);
        c->cur_lay = 0;
    }
    L(c).first_stage = 0;
    cudaFree(L(c).d_init_tiles);
    L(c).d_init_tiles = nullptr;
    L(c).n_init_tiles = 0;
    for (auto& b : c->deferred) release_block(c, b);
    c->deferred.clear();
}

}  // namespace

namespace {
int advance_impl(knc_ctx* c, int32_t fold, const double* dt_given);
}

int knc_advance(knc_ctx* c, int32_t fold) { return advance_impl(c, fold, nullptr); }

int knc_advance_dt(knc_ctx* c, int32_t fold, double dt) {
    if (!c || !(dt > 0.0)) return KNC_ERR_INVALID_ARGUMENT;
    return advance_impl(c, fold, &dt);
}

namespace {
int advance_impl(knc_ctx* c, int32_t fold, const double* dt_given) {
    if (!c || fold < 0) return KNC_ERR_INVALID_ARGUMENT;
    int r = KNC_OK;
    if ((r = check_ready(c))) return r;
    if ((r = rebuild_table(c))) return r;
    if ((r = update_ghost_geometry(c))) return r;
    if ((r = reset_status(c, true))) return r;
    const int per_step = c->hp.runge_kutta_order;
    // Adaptive dt (State::time_step, src/state.rs:151-160) normally costs a
    // full recovery pass before the fold. On a fixed mesh with a device model
    // the fold's first recovery reduces dl / a_max itself, every stage reads
    // dt = min x cfl from the device, ghost rows form their stage times there,
    // and the host learns dt (and advances the time) when the fold is done.
    const bool adaptive = !(c->hp.system == KNC_SYSTEM_RELATIVISTIC && !c->hp.adaptive_time_step);
    const bool ddt = !dt_given && adaptive && !c->mesh.moving() && c->model.kind != KNC_MODEL_HOST && fold > 0 &&
                     (int64_t)fold * per_step < 0xffff;
    double dt = 0.0;
    if (dt_given) {
        dt = *dt_given;
    } else if (ddt) {
        c->ddt = true;
        c->ddt_t0 = c->time;
        c->ddt_step = 0;
    } else if ((r = time_step_impl(c, &dt))) {
        return r;
    }
    auto finish_ddt = [&](int rr) {
        if (!c->ddt) return rr;
        c->ddt = false;
        if (rr == KNC_OK) {
            double dtmin;
            std::memcpy(&dtmin, &c->h_status->dt_bits, 8);
            const double dtv = dtmin * c->hp.cfl_number;
            double t = c->ddt_t0;
            for (int32_t k = 0; k < fold; ++k) t = step_times(per_step, t, dtv).end;
            c->time = t;
        }
        return rr;
    };
    const bool graph = c->batched && c->model.kind != KNC_MODEL_HOST && fold > 0 &&
                       c->stage_counter + (int64_t)fold * per_step < 0xffff;
    if (graph) {
        // One CUDA graph holds the whole fold: ghost, c2p, remap and update
        // launches of every stage, and the init launch of every block the
        // outer excision surface activates; a later fold with the same shape
        // only updates the executable graph's parameters (times, pointers)
        // instead of re-instantiating.
        std::vector<int> step_lay(fold, c->cur_lay);
        std::vector<char> step_init(fold, 0);
        if (c->mesh.moving() && (r = plan_fold(c, fold, dt, step_lay, step_init))) {
            c->failed = true;
            return r;
        }
        c->capturing = true;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int32_t k = 0; k < fold && r == KNC_OK; ++k) {
            if (c->cur_lay != step_lay[k]) {
                c->cur_lay = step_lay[k];
                L(c).first_stage = c->stage_counter;
            }
            if (step_init[k]) r = launch_activation(c);
            if (r == KNC_OK) r = rk_step(c, dt);
            if (c->ddt) ++c->ddt_step;
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
        c->capturing = false;
        if (r) {
            if (g) cudaGraphDestroy(g);
            c->failed = true;
            return finish_ddt(r);
        }
        if (ec != cudaSuccess) c->ddt = false;
        CK(ec);
        if (c->graph_exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(c->graph_exec, g, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(c->graph_exec);
                c->graph_exec = nullptr;
            }
        }
        cudaError_t ei = cudaSuccess;
        if (!c->graph_exec) ei = cudaGraphInstantiate(&c->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (ei == cudaSuccess) ei = cudaGraphLaunch(c->graph_exec, c->stream);
        if (ei != cudaSuccess) c->ddt = false;
        CK(ei);
        r = check_status(c);
        finish_fold(c);
        return finish_ddt(r);
    }
    for (int32_t k = 0; k < fold; ++k) {
        if (c->mesh.moving())
            if ((r = add_remove_blocks(c))) return r;
        if (c->stage_counter + per_step >= 0xffff) {
            if ((r = check_status(c))) return r;
            if ((r = reset_status(c, true))) return r;
        }
        r = rk_step(c, dt);
        if (c->ddt) ++c->ddt_step;
        if (r) return finish_ddt(r);
    }
    return finish_ddt(check_status(c));
}
}  // namespace

namespace {

// Chunks of consecutive slots for the host-state advance, about equal in
// zones, at most HOST_CHUNKS and at least one slot each: bounds[k] ..
// bounds[k + 1] - 1 are chunk k's slots. Fewer chunks start the downloads
// later, more pay more per copy and per launch chain; measured on the
// 4096 x 1024 wind (64 blocks), ms per step: 8 chunks 1.38, 10 1.35, 12
// 1.39, 16 1.40, 24 1.45.
constexpr int HOST_CHUNKS = 10;
// streams the chunks' launches are spread over (chunk k on k % HOST_STREAMS;
// at 10 chunks 1, 2, 3, 4 streams measured 1.36, 1.35, 1.35, 1.35 ms; at 16
// chunks 4 and 8 streams 1.40 and 1.42)
constexpr int HOST_STREAMS = 4;
// chunks whose uploads are issued before the next chunk's launches (at 10
// chunks 1 and 2 measured 1.36 and 1.35 ms; at 16 chunks 2 and 4 both 1.40)
constexpr int HOST_UPLOADS_AHEAD = 2;

std::vector<int> chunk_bounds(const Layout& l) {
    const int nb = (int)l.slot_index.size();
    const int G = std::min(HOST_CHUNKS, nb);
    std::vector<int> b{0};
    const int64_t total = l.zone_off[nb];
    for (int g = 1; g < G; ++g) {
        const int64_t target = total * g / G;
        int s = b.back() + 1;
        while (s < nb - (G - g) && l.zone_off[s] < target) ++s;   // a slot left for every later chunk
        b.push_back(s);
    }
    b.push_back(nb);
    return b;
}

// Whether every chunk boundary whose blocks exchange halo rows has the 2S
// rows on both sides that its shadow blocks copy (S stages per step).
bool chunks_fit(const Layout& l, int S) {
    const std::vector<int> cb = chunk_bounds(l);
    for (size_t k = 1; k + 1 < cb.size(); ++k) {
        const DevBlock& lo = l.tab_h[cb[k] - 1];
        const DevBlock& hi = l.tab_h[cb[k]];
        if (lo.P_out_nbr && (lo.nr < 2 * S || hi.nr < 2 * S)) return false;
    }
    return true;
}

// Independent chunks for the host-state advance (S stages per step). Each
// chunk boundary whose blocks exchange halo rows gets two shadow blocks of 2S
// rows: the first 2S rows of the block above it, for the chunk below, and
// the last 2S rows of the block below it, for the chunk above. In the chunk's
// own table the boundary block's halo rows come from its shadow and the
// shadow's from the boundary block. Each stage recovers all of a shadow's
// rows and updates those whose stencil lies inside the chunk and its shadow:
// rows [0, 2S - 2s - 2) of an upper shadow at stage s, rows [2s + 2, 2S) of a
// lower one. So the halo rows a chunk's blocks read are computed inside the
// chunk, from the same states with the same arithmetic as in the block they
// copy, and no chunk waits for another's launches. A shadow's rows that its
// stages do not update keep the step's initial state in both buffers
// (state_in_kernel), which recovers as at the first stage; they feed no
// update. A shadow's halo rows away from its chunk are never read.
int build_chunks(knc_ctx* c, int S) {
    Layout& l = L(c);
    if (l.sc_S == S) return KNC_OK;
    l.sc_S = 0;
    const int nb = (int)l.slot_index.size();
    l.sc_cb = chunk_bounds(l);
    const std::vector<int>& cb = l.sc_cb;
    const int G = (int)cb.size() - 1;
    std::vector<DevBlock> tab = l.tab_h;
    struct Shadow { int chunk, src, row0; bool upper; };
    std::vector<Shadow> sh;
    l.sc_up.assign(1, 0);
    for (int k = 1; k < G; ++k) {
        const int lo = cb[k] - 1, hi = cb[k];
        int64_t up = l.zone_off[hi];
        if (tab[lo].P_out_nbr) {
            sh.push_back({k - 1, hi, 0, true});
            sh.push_back({k, lo, tab[lo].nr - 2 * S, false});
            up += (int64_t)2 * S * tab[hi].nq;
        }
        l.sc_up.push_back(up);
    }
    l.sc_up.push_back(l.zone_off[nb]);
    size_t store = 0;
    for (const Shadow& x : sh) store += (size_t)(40 * S + 40) * tab[x.src].nq;
    if (store > l.sc_store_cap) {
        cudaFree(l.d_sc_store);
        l.d_sc_store = nullptr;
        CK(dalloc(&l.d_sc_store, store));
        l.sc_store_cap = store;
    }
    double* mem = l.d_sc_store;
    std::vector<std::vector<int>> of_chunk(G);
    for (size_t n = 0; n < sh.size(); ++n) {
        const Shadow& x = sh[n];
        const DevBlock src = l.tab_h[x.src];
        DevBlock d = src;
        const int64_t nq = src.nq, rows = 2 * S, o = x.row0;
        d.nr = (int32_t)rows;
        d.buf[0] = mem;
        d.buf[1] = mem + 5 * rows * nq;
        d.P = mem + 10 * rows * nq;
        d.P64 = mem + (15 * rows + 20) * nq;   // the mixed stage's FP64 primitives, like P
        mem += (5 * rows + 5 * (rows + 4) + 5 * rows + 5 * (rows + 4)) * nq;
        d.ar = src.ar + o * nq;
        d.aq = src.aq + o * (nq + 1);
        d.dv = src.dv + o * nq;
        d.rc = src.rc + o;
        d.rv = src.rv + o;
        d.ar_r = src.ar_r + o;
        d.aq_r = src.aq_r + o;
        d.dv_r = src.dv_r + o;
        d.dv_r32 = src.dv_r32 + o;
        d.rc32 = src.rc32 + o;
        d.shadow = 1;
        const int slot = nb + (int)n;
        if (x.upper) {   // above chunk x.chunk, whose last block is x.src - 1
            const int lo = x.src - 1;
            d.P_in_nbr = tab[lo].P;
            d.nr_in_nbr = tab[lo].nr;
            d.slot_in = lo;
            d.P_out_nbr = nullptr;
            d.nr_out_nbr = 0;
            d.slot_out = -1;
            tab[lo].P_out_nbr = d.P;
            tab[lo].nr_out_nbr = (int32_t)rows;
            tab[lo].slot_out = slot;
        } else {         // below chunk x.chunk, whose first block is x.src + 1
            const int hi = x.src + 1;
            d.P_out_nbr = tab[hi].P;
            d.nr_out_nbr = tab[hi].nr;
            d.slot_out = hi;
            d.P_in_nbr = nullptr;
            d.nr_in_nbr = 0;
            d.slot_in = -1;
            tab[hi].P_in_nbr = d.P;
            tab[hi].nr_in_nbr = (int32_t)rows;
            tab[hi].slot_in = slot;
        }
        tab.push_back(d);
        of_chunk[x.chunk].push_back((int)n);
    }
    // recovery tiles: per chunk its own blocks' (t.w = first zone of the
    // block in the whole-state arrays), then its shadows' (t.w = the zone of
    // the shadow's row 0 there)
    std::vector<int4> tiles;
    l.sc_tile_off.clear();
    l.sc_own_tiles.clear();
    const std::vector<int4>& own_tiles = l.tiles_h;
    for (int k = 0; k < G; ++k) {
        l.sc_tile_off.push_back((int)tiles.size());
        tiles.insert(tiles.end(), own_tiles.begin() + l.tile_off[cb[k]], own_tiles.begin() + l.tile_off[cb[k + 1]]);
        l.sc_own_tiles.push_back(l.tile_off[cb[k + 1]] - l.tile_off[cb[k]]);
        for (int n : of_chunk[k]) {
            const Shadow& x = sh[n];
            const int64_t w = l.zone_off[x.src] + (int64_t)x.row0 * tab[x.src].nq;
            for (int j0 = 0; j0 < tab[x.src].nq; j0 += TILE_Q) tiles.push_back(make_int4(nb + n, 0, j0, (int)w));
        }
    }
    l.sc_tile_off.push_back((int)tiles.size());
    // update strips: per chunk and stage its own blocks' short strips, then
    // its shadows' rows that stage updates
    std::vector<int4> strips;
    l.sc_strip_off.clear();
    for (int k = 0; k < G; ++k)
        for (int s = 0; s < S; ++s) {
            l.sc_strip_off.push_back((int)strips.size());
            strips.insert(strips.end(), l.sstrips_h.begin() + l.sstrip_off[cb[k]],
                          l.sstrips_h.begin() + l.sstrip_off[cb[k + 1]]);
            const int rows = 2 * S - 2 * s - 2;
            if (rows <= 0) continue;
            for (int n : of_chunk[k]) {
                const Shadow& x = sh[n];
                const int i0 = x.upper ? 0 : 2 * s + 2;
                for (int j0 = 0; j0 < tab[x.src].nq; j0 += STRIP_OUT)
                    strips.push_back(make_int4(nb + n, i0, j0, rows));
            }
        }
    l.sc_strip_off.push_back((int)strips.size());
    if ((int)tab.size() > l.sc_table_cap) {
        cudaFree(l.d_sc_table);
        l.d_sc_table = nullptr;
        CK(dalloc(&l.d_sc_table, tab.size()));
        l.sc_table_cap = (int)tab.size();
    }
    if ((int)tiles.size() > l.sc_tiles_cap) {
        cudaFree(l.d_sc_tiles);
        l.d_sc_tiles = nullptr;
        CK(dalloc(&l.d_sc_tiles, tiles.size()));
        l.sc_tiles_cap = (int)tiles.size();
    }
    if ((int)strips.size() > l.sc_strips_cap) {
        cudaFree(l.d_sc_strips);
        l.d_sc_strips = nullptr;
        CK(dalloc(&l.d_sc_strips, strips.size()));
        l.sc_strips_cap = (int)strips.size();
    }
    // (the chunk streams start after the library's stream)
    CK(cudaMemcpyAsync(l.d_sc_table, tab.data(), tab.size() * sizeof(DevBlock), cudaMemcpyHostToDevice, c->stream));
    if (!tiles.empty())
        CK(cudaMemcpyAsync(l.d_sc_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    if (!strips.empty())
        CK(cudaMemcpyAsync(l.d_sc_strips, strips.data(), strips.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           c->stream));
    l.sc_S = S;
    return KNC_OK;
}

int ensure_chunk_events(knc_ctx* c, size_t n) {
    while (c->ev_chunk.size() < n) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->ev_chunk.push_back(e);
    }
    return KNC_OK;
}

// One RK step with the state streamed between page-locked host memory and
// the device by chunks of blocks: hc_in / hs_in are uploaded before the
// step's first stage reads them, hc_out / hs_out downloaded after its last
// stage (either pair may be null; without an upload the step starts from the
// device state). Uploads (one copy direction), downloads (the other) and the
// chunks' launches run at the same time.
//
// Chunk k's launches go in order on a stream of their own: after the upload
// of its zones (and of the first 2S rows of the next chunk, which its upper
// shadow copies), state_in, then per stage the recovery of its blocks and
// shadows, the ghost rows at a mesh end, the update; then state_out into a
// separate staging area, which its download reads. No launch waits for
// another chunk (build_chunks), so chunk k's download starts once its own
// upload and six launches are done, and the last download follows the last
// upload by the same. Recoveries run in the inline form (the deferred list
// is per stage) and updates as short warp strips. Every zone of a block
// meets the arithmetic of rk_step, so states are bitwise those of
// knc_set_state + knc_advance + knc_get_state.
int stream_step(knc_ctx* c, double dt, const double* hc_in, const double* hs_in, double* hc_out,
                double* hs_out) {
    int r;
    StagePlan p[3];
    const int S = step_plan(c, dt, p);
    if ((r = build_chunks(c, S))) return r;
    const Layout& lay = L(c);
    const std::vector<int>& cb = lay.sc_cb;
    const int G = (int)cb.size() - 1;
    const int64_t total = lay.zone_off.back();
    GhostArgs g[3];
    StageArgs a[3];
    for (int s = 0; s < S; ++s)
        if ((r = prepare_stage(c, p[s].sel_in, p[s].sel_out, p[s].sel_base, p[s].w1, p[s].bf, p[s].t, dt, p[s].sub,
                               g[s], a[s])))
            return r;
    // staging: the step's input state (cons [total][4], then scalar [total]),
    // then its output state in the same layout, then per stage and mesh end
    // the ghost rows [5][2][nq], then (mixed) the same rows in FP64
    const int64_t gq = std::max(lay.nq_edge[0], lay.nq_edge[1]);
    if ((r = ensure_stage(c, 10 * (size_t)total + (size_t)S * 2 * 10 * gq * 2))) return r;
    const int NS = std::min(G, HOST_STREAMS);
    // events: uploads [0, G), downloads ready [G, 2 G), start, stream ends
    // [2 G + 1, 2 G + 2 + NS) (the last: ghost rows), ghost rows of stage s
    const size_t ev_start = (size_t)2 * G;
    const size_t ev_ghost = ev_start + 2 + NS;
    if ((r = ensure_chunk_events(c, ev_ghost + S))) return r;
    while ((int)c->kstreams.size() < NS + 1) {
        cudaStream_t st;
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        c->kstreams.push_back(st);
    }
    double* sc = c->d_stage;
    double* ss = c->d_stage + 4 * total;
    double* oc = c->d_stage + 5 * total;
    double* os = c->d_stage + 9 * total;
    if (!hc_in) {   // the device state into the input staging
        CK(launch_state_out(lay.d_table, lay.d_tiles, lay.ntiles, p[0].sel_in, sc, ss, c->stream));
        ++c->launches;
    }
    // every stream starts after the work already on the library's stream
    CK(cudaEventRecord(c->ev_chunk[ev_start], c->stream));
    for (int k = 0; k < NS; ++k) CK(cudaStreamWaitEvent(c->kstreams[k], c->ev_chunk[ev_start], 0));
    if (hc_in) CK(cudaStreamWaitEvent(c->h2d, c->ev_chunk[ev_start], 0));
    if (hc_out) CK(cudaStreamWaitEvent(c->d2h, c->ev_chunk[ev_start], 0));
    // The ghost rows of every stage depend only on the model and the stage
    // time: computed at once on a stream of their own into the staging area,
    // then copied into the edge block's halo rows just before the update of
    // the chunk at that mesh end, after its previous stage's update read them.
    cudaStream_t gst = c->kstreams[NS];
    CK(cudaStreamWaitEvent(gst, c->ev_chunk[ev_start], 0));
    double* gscr = c->d_stage + 10 * total;
    auto gscratch = [&](int s, int end) { return gscr + (size_t)(2 * s + end) * 10 * gq; };
    auto gscratch64 = [&](int s, int end) { return gscr + (size_t)(2 * S + 2 * s + end) * 10 * gq; };
    for (int s = 0; s < S; ++s) {
        GhostArgs ge = g[s];
        for (int end = 0; end < 2; ++end) {
            if (ge.P[end]) ge.P[end] = gscratch(s, end);
            if (ge.P64[end]) ge.P64[end] = gscratch64(s, end);
            ge.hp_list = nullptr;
            ge.row0[end] = 0;
            ge.nr_t[end] = -2;   // row stride nr_t + 4 = 2: the compact [5][2][nq]
        }
        CK(mixed(c) ? launch_ghost_mixed(ge, gst) : launch_ghost_f64(ge, gst));
        ++c->launches;
        CK(cudaEventRecord(c->ev_chunk[ev_ghost + s], gst));
    }
    CK(cudaEventRecord(c->ev_chunk[ev_start + 1 + NS], gst));
    auto upload = [&](int k) -> int {
        const int64_t z0 = lay.sc_up[k], nz = lay.sc_up[k + 1] - z0;
        if (nz > 0) {
            CK(cudaMemcpyAsync(sc + 4 * z0, hc_in + 4 * z0, 4 * nz * sizeof(double), cudaMemcpyHostToDevice,
                               c->h2d));
            CK(cudaMemcpyAsync(ss + z0, hs_in + z0, nz * sizeof(double), cudaMemcpyHostToDevice, c->h2d));
        }
        CK(cudaEventRecord(c->ev_chunk[k], c->h2d));
        return KNC_OK;
    };
    // Issue order: uploads HOST_UPLOADS_AHEAD chunks ahead of the chunk whose
    // launches are issued next, so that chunk 0's launches are queued while
    // its upload runs and the copy engine still always has the next upload.
    for (int k = 0; hc_in && k < std::min(G, HOST_UPLOADS_AHEAD); ++k)
        if ((r = upload(k))) return r;
    for (int k = 0; k < G; ++k) {
        if (hc_in && k + HOST_UPLOADS_AHEAD < G && (r = upload(k + HOST_UPLOADS_AHEAD))) return r;
        cudaStream_t st = c->kstreams[k % NS];
        if (hc_in) CK(cudaStreamWaitEvent(st, c->ev_chunk[k], 0));
        const int4* tiles = lay.d_sc_tiles + lay.sc_tile_off[k];
        const int ntiles = lay.sc_tile_off[k + 1] - lay.sc_tile_off[k];
        CK(launch_state_in(lay.d_sc_table, tiles, ntiles, p[0].sel_in, sc, ss, st));
        ++c->launches;
        for (int s = 0; s < S; ++s) {
            StageArgs y = a[s];
            y.blocks = lay.d_sc_table;
            y.tiles = tiles;
            y.ntiles = ntiles;
            // the update as warp strips of STREAM_STRIP_ROWS rows, whatever
            // the tuned form (every form gives the same state)
            y.strips = lay.d_sc_strips + lay.sc_strip_off[k * S + s];
            y.nstrips = lay.sc_strip_off[k * S + s + 1] - lay.sc_strip_off[k * S + s];
            y.tma = 0;
            // chunks run side by side: no shared list (each strip checks its
            // own stencil and updates its zones with FP64 faces itself)
            y.hp_list = nullptr;
            y.hp_count = nullptr;
            y.hp_claim = nullptr;
            y.hp_count_next = nullptr;
            y.hp_claim_next = nullptr;
            y.hp_cap = 0;
            y.high = nullptr;
            y.high_count = nullptr;
            y.high_count_next = nullptr;
            y.high_cap = 0;
            CK(mixed(c) ? launch_c2p_mixed(y, st) : launch_c2p_f64(y, st));
            ++c->launches;
            for (int end = 0; end < 2; ++end) {
                if (k != (end ? G - 1 : 0) || !g[s].P[end]) continue;
                CK(cudaStreamWaitEvent(st, c->ev_chunk[ev_ghost + s], 0));
                CK(launch_halo_rows(gscratch(s, end), g[s].P[end], g[s].nq[end], g[s].nr_t[end], g[s].row0[end],
                                    mixed(c) ? 4 : 8, st));
                ++c->launches;
                if (g[s].P64[end]) {
                    // mixed: the rows in FP64 too (zone_hp reads those above the split)
                    CK(launch_halo_rows(gscratch64(s, end), g[s].P64[end], g[s].nq[end], g[s].nr_t[end],
                                        g[s].row0[end], 8, st));
                    ++c->launches;
                }
            }
            CK(mixed(c) ? launch_update_mixed(y, st) : launch_update_f64(y, st));
            ++c->launches;
        }
        if (hc_out) {
            const int64_t z0 = lay.zone_off[cb[k]], nz = lay.zone_off[cb[k + 1]] - z0;
            CK(launch_state_out(lay.d_sc_table, tiles, lay.sc_own_tiles[k], p[S - 1].sel_out, oc, os, st));
            ++c->launches;
            CK(cudaEventRecord(c->ev_chunk[G + k], st));
            CK(cudaStreamWaitEvent(c->d2h, c->ev_chunk[G + k], 0));
            CK(cudaMemcpyAsync(hc_out + 4 * z0, oc + 4 * z0, 4 * nz * sizeof(double), cudaMemcpyDeviceToHost,
                               c->d2h));
            CK(cudaMemcpyAsync(hs_out + z0, os + z0, nz * sizeof(double), cudaMemcpyDeviceToHost, c->d2h));
        }
    }
    // the library's stream continues after every chunk stream, the ghost rows
    // and the downloads
    for (int k = 0; k < NS; ++k) {
        CK(cudaEventRecord(c->ev_chunk[ev_start + 1 + k], c->kstreams[k]));
        CK(cudaStreamWaitEvent(c->stream, c->ev_chunk[ev_start + 1 + k], 0));
    }
    CK(cudaStreamWaitEvent(c->stream, c->ev_chunk[ev_start + 1 + NS], 0));
    if (hc_out) {
        CK(cudaEventRecord(c->ev_chunk[ev_start], c->d2h));
        CK(cudaStreamWaitEvent(c->stream, c->ev_chunk[ev_start], 0));
    }
    c->zone_updates += lay.nzones;
    finish_step(c, dt);
    return KNC_OK;
}

int advance_host_streamed(knc_ctx* c, const double* cons_in, const double* scalar_in, double* cons_out,
                          double* scalar_out, int32_t fold) {
    int r;
    if ((r = update_ghost_geometry(c))) return r;
    if ((r = reset_status(c, true))) return r;
    double dt = 0.0;
    if ((r = time_step_impl(c, &dt))) return r;
    c->failed = false;
    const int per_step = c->hp.runge_kutta_order;
    for (int32_t k = 0; k < fold; ++k) {
        if (c->stage_counter + per_step >= 0xffff) {
            if ((r = check_status(c))) return r;
            if ((r = reset_status(c, true))) return r;
        }
        const bool first = k == 0, last = k == fold - 1;
        if (first || last)
            r = stream_step(c, dt, first ? cons_in : nullptr, first ? scalar_in : nullptr, last ? cons_out : nullptr,
                            last ? scalar_out : nullptr);
        else
            r = rk_step(c, dt);
        if (r) return r;
    }
    return check_status(c);
}

}  // namespace

int knc_advance_host(knc_ctx* c, const double* cons_in, const double* scalar_in, double* cons_out,
                     double* scalar_out, int32_t fold) {
    if (!c || !cons_in || !scalar_in || !cons_out || !scalar_out || fold < 0) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = check_ready(c))) return r;
    if (c->mesh.moving())
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT,
                       "advance_host: moving excision surfaces change the block set inside the fold; "
                       "use knc_advance and knc_get_block");
    if ((r = rebuild_table(c))) return r;
    const bool adaptive = !(c->hp.system == KNC_SYSTEM_RELATIVISTIC && !c->hp.adaptive_time_step);
    const bool pinned = device_view(cons_in) && device_view(scalar_in) && device_view(cons_out) &&
                        device_view(scalar_out);
    // (the chunks update as warp strips, which need a polar grid)
    const bool streamed = pinned && fold > 0 && !adaptive && !c->fused && L(c).nremap == 0 &&
                          c->model.kind != KNC_MODEL_HOST && c->mesh.p.num_polar_zones > 1 &&
                          chunks_fit(L(c), c->hp.runge_kutta_order);
    if (!streamed) {
        // whole-state copies around the fold
        if ((r = knc_set_state(c, cons_in, scalar_in))) return r;
        if ((r = advance_impl(c, fold, nullptr))) return r;
        return knc_get_state(c, cons_out, scalar_out);
    }
    r = advance_host_streamed(c, cons_in, scalar_in, cons_out, scalar_out, fold);
    // the caller's buffers are free again when the call returns, on failure too
    cudaStreamSynchronize(c->h2d);
    cudaStreamSynchronize(c->d2h);
    for (cudaStream_t st : c->kstreams) cudaStreamSynchronize(st);
    cudaStreamSynchronize(c->stream);
    if (r) c->failed = true;
    return r;
}

int knc_set_profiling(knc_ctx* c, int32_t on) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    drain_profile(c);
    for (int k = 0; k < KNC_KERNEL_KINDS; ++k) {
        c->prof_ms[k] = 0.0;
        c->prof_count[k] = 0;
    }
    c->profiling = on != 0;
    return KNC_OK;
}

int knc_kernel_times(knc_ctx* c, double* ms, int64_t* launches) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    drain_profile(c);
    for (int k = 0; k < KNC_KERNEL_KINDS; ++k) {
        if (ms) ms[k] = c->prof_ms[k];
        if (launches) launches[k] = c->prof_count[k];
    }
    return KNC_OK;
}

int knc_set_device(int32_t device) {
    return cudaSetDevice(device) == cudaSuccess ? KNC_OK : KNC_ERR_CUDA;
}

int knc_device_count(int32_t* count) {
    if (!count) return KNC_ERR_INVALID_ARGUMENT;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return KNC_OK;
}

int knc_host_alloc(size_t bytes, void** ptr) {
    if (!ptr || bytes == 0) return KNC_ERR_INVALID_ARGUMENT;
    if (cudaHostAlloc(ptr, bytes, cudaHostAllocDefault) != cudaSuccess) return KNC_ERR_OUT_OF_MEMORY;
    return KNC_OK;
}

int knc_host_free(void* ptr) {
    if (!ptr) return KNC_OK;
    return cudaFreeHost(ptr) == cudaSuccess ? KNC_OK : KNC_ERR_CUDA;
}

int knc_set_precision(knc_ctx* c, int32_t precision) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (precision != KNC_PRECISION_FP64 && precision != KNC_PRECISION_MIXED)
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    c->precision = precision;
    return KNC_OK;
}

int knc_set_c2p_guess(knc_ctx* c, int32_t guess, const float* w, size_t n) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (guess == KNC_GUESS_PLAIN) {
        c->guess = guess;
        return KNC_OK;
    }
    if (guess != KNC_GUESS_MLP || !w || n != (size_t)KNC_MLP_NUM_PARAMS)
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "MLP guess needs %d weights", KNC_MLP_NUM_PARAMS);
    if (!c->d_mlp) CK(dalloc(&c->d_mlp, (size_t)KNC_MLP_NUM_PARAMS));
    CK(cudaMemcpyAsync(c->d_mlp, w, n * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->guess = guess;
    return KNC_OK;
}

int knc_zone_updates(const knc_ctx* c, int64_t* n) {
    if (!c || !n) return KNC_ERR_INVALID_ARGUMENT;
    *n = c->zone_updates;
    return KNC_OK;
}

int knc_set_tuning(knc_ctx* c, const knc_tuning* t) {
    if (!c || !t) return KNC_ERR_INVALID_ARGUMENT;
    if (t->update_form < KNC_UPDATE_TILE || t->update_form > KNC_UPDATE_STRIP)
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "unknown update form %d", t->update_form);
    const bool strip = t->update_form == KNC_UPDATE_STRIP;
    if (strip ? (t->tile_rows < 4 || t->tile_rows > 64)
              : (t->tile_rows != 4 && t->tile_rows != 8 && t->tile_rows != 16))
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "tile_rows must be 4, 8 or 16 (tiles) or 4..64 (strips)");
    if (strip && c->mesh.p.num_polar_zones == 1)
        return set_msg(c, KNC_ERR_UNSUPPORTED, "warp strips need num_polar_zones > 1");
    if (t->ctas_per_sm < 0) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "ctas_per_sm must be >= 0");
    if (t->recovery_form != KNC_RECOVERY_INLINE && t->recovery_form != KNC_RECOVERY_DEFERRED)
        return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "unknown recovery form %d", t->recovery_form);
    if (t->fused && !c->coop)
        return set_msg(c, KNC_ERR_UNSUPPORTED, "the device has no cooperative launch (fused stage)");
    c->utr = t->tile_rows;
    c->fused = t->fused ? 1 : 0;
    c->ctas_per_sm = t->ctas_per_sm;
    // the fused stage stages its tiles itself (no tensor-copy form)
    c->uform = t->fused && t->update_form == KNC_UPDATE_TILE_TMA ? KNC_UPDATE_TILE : t->update_form;
    c->rform = t->recovery_form;
    return KNC_OK;
}

int knc_get_tuning(const knc_ctx* c, knc_tuning* t) {
    if (!c || !t) return KNC_ERR_INVALID_ARGUMENT;
    t->tile_rows = c->utr;
    t->fused = c->fused;
    t->ctas_per_sm = c->ctas_per_sm;
    t->update_form = c->uform;
    t->recovery_form = c->rform;
    return KNC_OK;
}

int knc_autotune(knc_ctx* c, int32_t reps, knc_tuning* best_out, double* ms_out) {
    if (!c || reps < 1) return KNC_ERR_INVALID_ARGUMENT;
    int r;
    if ((r = check_ready(c))) return r;
    if ((r = rebuild_table(c))) return r;
    if ((r = update_ghost_geometry(c))) return r;
    if ((r = reset_status(c, true))) return r;
    double dt;
    if ((r = time_step_impl(c, &dt))) return r;
    DevStatus saved;
    CK(cudaMemcpy(&saved, c->d_status, sizeof(saved), cudaMemcpyDeviceToHost));
    const knc_tuning keep = {c->utr, c->fused, c->ctas_per_sm, c->uform, c->rform};
    std::vector<knc_tuning> cands;
    // strip heights: powers of two and some between (the last wave of
    // resident warps fills differently; measured on the 4096 x 1024 wind the
    // spread from 8 to 20 rows is within 2%)
    if (c->mesh.p.num_polar_zones > 1)
        for (int sr : {4, 8, 10, 12, 16, 20, 24, 32, 64})
            for (int mb : {4, 5, 6})
                if (mixed(c) || mb == 4) cands.push_back({sr, 0, mb, KNC_UPDATE_STRIP});
    // The fused stages (one cooperative launch per stage) only for solvers
    // that launch their stages from the host one by one, the way candidates
    // are timed: inside a batched solver's captured folds, where the
    // separate launches' gaps are hidden, every fused form measured slower
    // than the separate launches (by 2-8% for the fused deferring stage)
    const bool offer_fused = c->coop && !c->batched;
    for (int tr : {4, 8, 16}) {
        cands.push_back({tr, 0, 0, KNC_UPDATE_TILE});
        // tensor-copy staging (used where every block allows it)
        if (mixed(c)) cands.push_back({tr, 0, 0, KNC_UPDATE_TILE_TMA});
        if (!offer_fused) continue;
        c->utr = tr;
        int per_sm = 1;
        const bool mlp = c->guess == KNC_GUESS_MLP && c->d_mlp;
        CK(mixed(c) ? fused_max_ctas_mixed(mlp, tr, &per_sm)
                    : fused_max_ctas_f64(mlp && c->hp.system == KNC_SYSTEM_RELATIVISTIC, tr, &per_sm));
        for (int k = 1; k <= per_sm && k <= 8; ++k) cands.push_back({tr, 1, k, KNC_UPDATE_TILE});
    }
    if (offer_fused && c->mesh.p.num_polar_zones > 1) {
        // the fused stage with warp strips in its update phase (CTAs of 9 warps)
        int per_sm = 1;
        const bool mlp = c->guess == KNC_GUESS_MLP && c->d_mlp;
        CK(mixed(c) ? fused_strip_max_ctas_mixed(mlp, &per_sm)
                    : fused_max_ctas_f64(mlp && c->hp.system == KNC_SYSTEM_RELATIVISTIC, 8, &per_sm));
        for (int sr : {8, 16, 32})
            for (int k = 1; k <= per_sm && k <= 8; ++k) cands.push_back({sr, 1, k, KNC_UPDATE_STRIP});
        if (mixed(c)) {
            // with the deferring recovery (the separate form's five launches in one)
            CK(fused_deferred_max_ctas_mixed(mlp, 5, &per_sm));
            // (k = 1: one CTA of 20 warps per SM)
            for (int sr : {8, 12, 16, 32}) {
                cands.push_back({sr, 1, 1, KNC_UPDATE_STRIP, KNC_RECOVERY_DEFERRED});
                for (int k = std::max(2, per_sm - 1); k <= per_sm && k <= 8; ++k)
                    cands.push_back({sr, 1, k, KNC_UPDATE_STRIP, KNC_RECOVERY_DEFERRED});
            }
        }
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    knc_tuning best = keep;
    double best_ms = -1.0;
    const bool prof = c->profiling;
    c->profiling = false;
    // the launch shapes with inline recovery, then (mixed, separate) the best
    // of them with the deferred dense recovery
    for (size_t ci = 0; ci < cands.size(); ++ci) {
        const knc_tuning t = cands[ci];
        c->utr = t.tile_rows;
        c->fused = t.fused;
        c->ctas_per_sm = t.ctas_per_sm;
        c->uform = t.update_form;
        c->rform = t.recovery_form;
        // a fresh start for the deferred-recovery counters of every candidate
        CK(cudaMemsetAsync(c->d_status->high_count, 0, sizeof(c->d_status->high_count), c->stream));
        CK(cudaMemsetAsync(c->d_status->hp_count, 0, sizeof(c->d_status->hp_count) + sizeof(c->d_status->hp_claim),
                           c->stream));
        if ((r = rebuild_table(c))) break;
        if (t.update_form == KNC_UPDATE_TILE_TMA && !L(c).tma_ok) continue;
        // the first stage reads buf[cur] and writes buf[1 - cur]: the state stays
        if ((r = run_stage(c, c->cur, 1 - c->cur, -1, 1.0, 0.0, c->time, dt, 0))) break;
        CK(cudaEventRecord(e0, c->stream));
        for (int k = 0; k < reps && r == KNC_OK; ++k) r = run_stage(c, c->cur, 1 - c->cur, -1, 1.0, 0.0, c->time, dt, 0);
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        if (r) break;
        if ((r = check_status(c))) break;
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        const double per = (double)ms / reps;
        if (best_ms < 0.0 || per < best_ms) {
            best_ms = per;
            best = t;
        }
        c->stage_counter = 0;
        if (ci + 1 == cands.size() && mixed(c) && !best.fused && best.recovery_form == KNC_RECOVERY_INLINE) {
            knc_tuning d = best;
            d.recovery_form = KNC_RECOVERY_DEFERRED;
            cands.push_back(d);
        }
    }
    c->profiling = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    saved.bar_count = 0;
    saved.bar_abort = 0;
    saved.high_count[0] = 0;
    saved.high_count[1] = 0;
    CK(cudaMemcpy(c->d_status, &saved, sizeof(saved), cudaMemcpyHostToDevice));
    c->stage_counter = 0;
    c->bar_epoch = 0;
    c->utr = best.tile_rows;
    c->fused = best.fused;
    c->ctas_per_sm = best.ctas_per_sm;
    c->uform = best.update_form;
    c->rform = best.recovery_form;
    if (r) {
        c->failed = false;
        return r;
    }
    if ((r = rebuild_table(c))) return r;
    if (best_out) *best_out = best;
    if (ms_out) *ms_out = best_ms;
    return KNC_OK;
}

int knc_set_batched(knc_ctx* c, int32_t graph) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    c->batched = graph ? 1 : 0;
    return KNC_OK;
}

int knc_set_wait_test(knc_ctx* c, int32_t polls, int32_t unreachable) {
    if (!c || polls < 0) return KNC_ERR_INVALID_ARGUMENT;
    c->wait_polls = polls;
    c->wait_unreachable = unreachable ? 1 : 0;
    return KNC_OK;
}

int knc_set_mixed_w_split(knc_ctx* c, double w_split) {
    if (!c || !(w_split >= 1.0)) return KNC_ERR_INVALID_ARGUMENT;
    c->w_split = w_split;
    return KNC_OK;
}

int knc_synchronize(knc_ctx* c) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

int knc_c2p_stats(knc_ctx* c, int64_t* zones, int64_t* it64, int64_t* it32, int64_t* fb) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    DevStatus s;
    CK(cudaMemcpyAsync(&s, c->d_status, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (zones) *zones = (int64_t)s.c2p_zones;
    if (it64) *it64 = (int64_t)s.iters_fp64;
    if (it32) *it32 = (int64_t)s.iters_fp32;
    if (fb) *fb = (int64_t)s.fallbacks;
    return KNC_OK;
}

int knc_reset_c2p_stats(knc_ctx* c) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    return reset_status(c, false);
}

int knc_launch_count(const knc_ctx* c, int64_t* launches) {
    if (!c || !launches) return KNC_ERR_INVALID_ARGUMENT;
    *launches = c->launches;
    return KNC_OK;
}

int knc_sample_pairs(knc_ctx* c, int32_t stride, double* out, int64_t capacity, int64_t* written) {
    if (!c || !out || stride <= 0 || capacity <= 0) return KNC_ERR_INVALID_ARGUMENT;
    if (c->hp.system != KNC_SYSTEM_RELATIVISTIC)
        return set_msg(c, KNC_ERR_UNSUPPORTED, "pairs are defined for relativistic hydro");
    if (c->blocks.empty()) return set_msg(c, KNC_ERR_INVALID_ARGUMENT, "no blocks");
    int r;
    if ((r = rebuild_table(c))) return r;
    double* d_out = nullptr;
    unsigned long long* d_cnt = nullptr;
    CK(dalloc(&d_out, (size_t)capacity * 8));
    cudaError_t e = dalloc(&d_cnt, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, 8, c->stream);
    if (e == cudaSuccess)
        e = launch_sample_pairs(L(c).d_table, L(c).d_tiles, L(c).ntiles, c->cur, stride, c->hp.gamma_law_index, d_out,
                                capacity, d_cnt, c->stream);
    ++c->launches;
    unsigned long long cnt = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&cnt, d_cnt, 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    const int64_t nw = std::min<int64_t>((int64_t)cnt, capacity);
    if (e == cudaSuccess && nw > 0) e = cudaMemcpy(out, d_out, (size_t)nw * 8 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_cnt);
    CK(e);
    if (written) *written = nw;
    return KNC_OK;
}

int knc_mark(knc_ctx* c, int32_t slot) {
    if (!c || slot < 0 || slot >= 8) return KNC_ERR_INVALID_ARGUMENT;
    if (!c->marks[slot]) CK(cudaEventCreate(&c->marks[slot]));
    CK(cudaEventRecord(c->marks[slot], c->stream));
    return KNC_OK;
}

int knc_elapsed_ms(knc_ctx* c, int32_t a, int32_t b, double* ms) {
    if (!c || !ms || a < 0 || a >= 8 || b < 0 || b >= 8 || !c->marks[a] || !c->marks[b])
        return KNC_ERR_INVALID_ARGUMENT;
    CK(cudaEventSynchronize(c->marks[b]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, c->marks[a], c->marks[b]));
    *ms = f;
    return KNC_OK;
}

namespace {
// FP64 recovery of one block's tiles into its (double) primitive array.
int recover_block_f64(knc_ctx* c, int32_t index) {
    int r;
    if ((r = check_ready(c))) return r;
    if ((r = rebuild_table(c))) return r;
    if ((r = reset_status(c, true))) return r;
    StageArgs a = base_args(c);
    a.mlp = nullptr;
    a.stage = c->stage_counter++;
    a.sel_in = c->cur;
    a.sel_out = c->cur;
    const std::vector<int32_t>& si = L(c).slot_index;
    const int slot = (int)(std::find(si.begin(), si.end(), index) - si.begin());
    a.tiles = L(c).d_tiles + L(c).tile_off[slot];
    a.ntiles = L(c).tile_off[slot + 1] - L(c).tile_off[slot];
    CK(launch_c2p_f64(a, c->stream));
    ++c->launches;
    return check_status(c);
}
}  // namespace

int knc_get_products(knc_ctx* c, int32_t index, double* radial_vertices, double* polar_vertices,
                     double* primitive, double* scalar) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return set_msg(c, KNC_ERR_NO_BLOCK, "no block %d", index);
    const BlockH& b = it->second;
    if (radial_vertices) std::memcpy(radial_vertices, b.geom.rv.data(), b.geom.rv.size() * sizeof(double));
    if (polar_vertices) std::memcpy(polar_vertices, b.geom.qv.data(), b.geom.qv.size() * sizeof(double));
    if (!primitive && !scalar) return KNC_OK;
    int r;
    if ((r = recover_block_f64(c, index))) return r;
    const size_t n = (size_t)(b.nr * b.nq);
    if ((r = ensure_stage(c, 5 * n))) return r;
    CK(launch_products(b.P, b.buf[c->cur], c->d_stage, c->d_stage + 4 * n, b.nr, b.nq, c->stream));
    ++c->launches;
    if (primitive) CK(cudaMemcpyAsync(primitive, c->d_stage, 4 * n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (scalar) CK(cudaMemcpyAsync(scalar, c->d_stage + 4 * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

int knc_get_primitives(knc_ctx* c, int32_t index, double* prim) {
    if (!c || !prim) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return set_msg(c, KNC_ERR_NO_BLOCK, "no block %d", index);
    int r;
    if ((r = check_ready(c))) return r;
    if ((r = rebuild_table(c))) return r;
    if ((r = reset_status(c, true))) return r;
    StageArgs a = base_args(c);
    a.mlp = nullptr;
    a.stage = c->stage_counter++;
    a.sel_in = c->cur;
    a.sel_out = c->cur;
    // FP64 recovery of this block's tiles only, double primitives
    const std::vector<int32_t>& si = L(c).slot_index;
    const int slot = (int)(std::find(si.begin(), si.end(), index) - si.begin());
    a.tiles = L(c).d_tiles + L(c).tile_off[slot];
    a.ntiles = L(c).tile_off[slot + 1] - L(c).tile_off[slot];
    CK(launch_c2p_f64(a, c->stream));
    ++c->launches;
    if ((r = check_status(c))) return r;
    const BlockH& b = it->second;
    const size_t n = (size_t)(b.nr * b.nq);
    if ((r = ensure_stage(c, 5 * n))) return r;
    CK(launch_prims_to_aos(b.P, c->d_stage, b.nr, b.nq, c->stream));
    ++c->launches;
    CK(cudaMemcpyAsync(prim, c->d_stage, 5 * n * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KNC_OK;
}

}  // extern "C"
