// Host orchestration of the device-resident world (the GB300 counterpart of pe_intf::World).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <map>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <tuple>
#include <utility>
#include <vector>
#include "pe_host.h"
#include "pe_kernels.cuh"

namespace pe {

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};
#define PE_CK(x)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));    \
    } while (0)

// Counts device-array reallocations in this process: a captured step graph holds the addresses it
// was captured with, so any reallocation since then sends the step back through a new capture.
inline std::atomic<unsigned long long>& dbuf_generation() {
    static std::atomic<unsigned long long> g{0};
    return g;
}
template <class T> struct DBuf {   // device array that grows on demand
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { if (p) cudaFree(p); }
    void ensure(size_t want, bool keep = false) {
        if (want <= n && p) return;
        size_t cap = want < 16 ? 16 : want;
        T* q = nullptr;
        PE_CK(cudaMalloc(&q, cap * sizeof(T)));
        if (keep && p && n) PE_CK(cudaMemcpy(q, p, n * sizeof(T), cudaMemcpyDeviceToDevice));
        if (p) cudaFree(p);
        p = q;
        n = cap;
        dbuf_generation()++;
    }
};

// kernel groups for per-kernel device time (profiling mode)
enum KernelId { K_INTEGRATE = 0, K_BP_KEYS, K_RADIX, K_SCAN, K_BP_GATHER, K_BP_SWEEP, K_BP_AXIS, K_NP_BUCKET, K_NP, K_NP_SAT,
                K_SI_SETUP, K_ISLAND, K_SI_SERIAL, K_SI_COLOR, K_GC_COLOR, K_GC_SOLVE, K_SI_MISC, K_MISC, K_COUNT };
inline const char* kernel_name(int k) {
    static const char* n[K_COUNT] = {"integrate", "bp_keys", "radix_sort", "scan", "bp_gather", "bp_sweep", "bp_axis",
                                     "np_bucket", "narrowphase", "np_sat", "si_setup", "islands", "si_serial", "si_colored",
                                     "big_island_color", "big_island_solve", "si_misc", "misc"};
    return k >= 0 && k < K_COUNT ? n[k] : "";
}

class WorldBase {
public:
    virtual void set_profiling(bool on) = 0;
    virtual void kernel_stats(double* ms, long long* launches) = 0;
    virtual ~WorldBase() {}
    virtual int real_bits() const = 0;
    virtual void set_shapes(int S, const int* type, const double* param, const int* vbeg, const int* vcnt, const int* fbeg,
                            const int* fcnt, int HV, const double* hv, int HF, const int* foff, const int* fidx) = 0;
    virtual void set_bodies(int n, const int* shape, const int* flags, const double* mass, const double* fr,
                            const double* re, const double* ld, const double* ad, const double* o, const double* b,
                            const double* v, const double* w) = 0;
    virtual void set_compounds(const int* cbeg, const int* ccnt, int C, const int* cshape, const double* corg,
                               const double* cbas, const double* cratio, const double* local_inertia, double* centroid) = 0;
    virtual void set_joints(int n, const int* type, const int* body, const int* flag, const double* param) = 0;
    virtual void set_ignore_pairs(int n, const int* pairs) = 0;
    virtual void set_scenes(int n, const int* off) = 0;
    virtual void set_params(double dt, double gx, double gy, double gz, int iters) = 0;
    virtual void set_margin(double m) = 0;
    virtual Tuning& tuning() = 0;
    virtual void step(int n, int mode) = 0;
    virtual void integrate() = 0;
    virtual int broadphase() = 0;
    virtual void narrowphase() = 0;
    virtual void solve(int mode) = 0;
    virtual int n_bodies() const = 0;
    virtual void get_state(double* o, double* b, double* v, double* w, double* mn, double* mx, double* iw) = 0;
    virtual void set_state(const double* o, const double* b, const double* v, const double* w, const double* mn,
                           const double* mx, const double* iw) = 0;
    // the same in single precision (pe::Real of the reference's default build)
    virtual void get_state(float* o, float* b, float* v, float* w, float* mn, float* mx, float* iw) = 0;
    virtual void set_state(const float* o, const float* b, const float* v, const float* w, const float* mn,
                           const float* mx, const float* iw) = 0;
    virtual void get_axes(int* a) = 0;
    virtual void set_axes(const int* a) = 0;
    virtual int n_pairs() const = 0;
    virtual void get_pairs(int* p) = 0;
    virtual void set_pairs(int n, const int* p) = 0;
    virtual int n_results() const = 0;
    virtual void get_results(int* a, int* b, int* ps, double* fr, double* re, double* slots) = 0;
    virtual void set_results(int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                             const double* slots) = 0;
    virtual void phase_times(double* ms, bool reset) = 0;
    virtual void last_counts(int* c) = 0;
    virtual void sync() = 0;
    // steps replay a captured CUDA graph of their device part (on by default)
    virtual void set_step_graphs(bool on) = 0;
    virtual bool step_graphs() const = 0;
    // serving: replace the scene list by the kept scenes (old indices, in the new order) followed by
    // the added ones, keeping the kept scenes' bodies, sweep axes and contact-result pools on the device
    virtual void repack(const int* keep, int n_keep, const SceneData* const* adds, int n_add) = 0;
    virtual const std::vector<int>& scene_body_offsets() const = 0;
    virtual void get_state_range(int first, int count, double* o, double* b, double* v, double* w) = 0;
    std::string err;
};

template <class R> class World : public WorldBase {
public:
    explicit World(int device);
    ~World() override;
    using WorldBase::set_profiling;
    int real_bits() const override { return sizeof(R) * 8; }
    void set_shapes(int S, const int* type, const double* param, const int* vbeg, const int* vcnt, const int* fbeg,
                    const int* fcnt, int HV, const double* hv, int HF, const int* foff, const int* fidx) override;
    void set_bodies(int n, const int* shape, const int* flags, const double* mass, const double* fr, const double* re,
                    const double* ld, const double* ad, const double* o, const double* b, const double* v,
                    const double* w) override;
    void set_compounds(const int* cbeg, const int* ccnt, int C, const int* cshape, const double* corg, const double* cbas,
                       const double* cratio, const double* local_inertia, double* centroid) override;
    void set_joints(int n, const int* type, const int* body, const int* flag, const double* param) override;
    void set_ignore_pairs(int n, const int* pairs) override;
    void set_scenes(int n, const int* off) override;
    void set_params(double dt, double gx, double gy, double gz, int iters) override;
    void set_margin(double m) override { margin_ = static_cast<R>(m); }
    Tuning& tuning() override { return tun_; }
    void step(int n, int mode) override;
    void integrate() override;
    int broadphase() override;
    void narrowphase() override;
    void solve(int mode) override;
    int n_bodies() const override { return N_; }
    void get_state(double* o, double* b, double* v, double* w, double* mn, double* mx, double* iw) override {
        get_state_t(o, b, v, w, mn, mx, iw);
    }
    void set_state(const double* o, const double* b, const double* v, const double* w, const double* mn, const double* mx,
                   const double* iw) override {
        set_state_t(o, b, v, w, mn, mx, iw);
    }
    void get_state(float* o, float* b, float* v, float* w, float* mn, float* mx, float* iw) override { get_state_t(o, b, v, w, mn, mx, iw); }
    void set_state(const float* o, const float* b, const float* v, const float* w, const float* mn, const float* mx,
                   const float* iw) override {
        set_state_t(o, b, v, w, mn, mx, iw);
    }
    template <class T> void get_state_t(T* o, T* b, T* v, T* w, T* mn, T* mx, T* iw);
    template <class T> void set_state_t(const T* o, const T* b, const T* v, const T* w, const T* mn, const T* mx, const T* iw);
    void get_axes(int* a) override;
    void set_axes(const int* a) override;
    int n_pairs() const override { return P_; }
    void get_pairs(int* p) override;
    void set_pairs(int n, const int* p) override;
    int n_results() const override { return R_; }
    void get_results(int* a, int* b, int* ps, double* fr, double* re, double* slots) override;
    void set_results(int n, const int* a, const int* b, const int* ps, const double* fr, const double* re,
                     const double* slots) override;
    void phase_times(double* ms, bool reset) override;
    void last_counts(int* c) override;
    void sync() override { PE_CK(cudaStreamSynchronize(st_)); }
    void set_step_graphs(bool on) override { graphs_ = on; }
    bool step_graphs() const override { return graphs_; }
    void repack(const int* keep, int n_keep, const SceneData* const* adds, int n_add) override;
    const std::vector<int>& scene_body_offsets() const override { return h_scene_off_; }
    void get_state_range(int first, int count, double* o, double* b, double* v, double* w) override;
    void set_profiling(bool on) override {
        resolve_prof();
        if (on && !prof_) for (int k = 0; k < K_COUNT; k++) { kms_[k] = 0; klaunch_[k] = 0; }
        prof_ = on;
    }
    void kernel_stats(double* ms, long long* launches) override {
        resolve_prof();
        for (int k = 0; k < K_COUNT; k++) { ms[k] = kms_[k]; launches[k] = klaunch_[k]; }
    }

private:
    // every kernel of the step goes through here: counts launches, and in profiling mode
    // brackets the launch with events on the world's stream
    template <class Kern, class... A> void launch(int id, int g, Kern kern, A... args) { launch_smem(id, g, kBlock, 0, kern, args...); }
    template <class Kern, class... A> void launch_block(int id, int g, int block, Kern kern, A... args) {
        launch_smem(id, g, block, 0, kern, args...);
    }
    template <class Kern, class... A> void launch_smem(int id, int g, int block, size_t smem, Kern kern, A... args) {
        if (g <= 0) return;
        klaunch_[id]++;
        step_launches_++;
        cudaStream_t s = cur_ ? cur_ : st_;   // a side stream while a fork is open (fork_streams)
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (prof_) {
            if (ev_pool_.size() < 2) { cudaEvent_t a, b; PE_CK(cudaEventCreate(&a)); PE_CK(cudaEventCreate(&b)); ev_pool_.push_back(a); ev_pool_.push_back(b); }
            e0 = ev_pool_.back(); ev_pool_.pop_back();
            e1 = ev_pool_.back(); ev_pool_.pop_back();
            PE_CK(cudaEventRecord(e0, s));
        }
        kern<<<g, block, smem, s>>>(args...);
        if (prof_) {
            PE_CK(cudaEventRecord(e1, s));
            pending_.push_back({id, e0, e1});
        }
    }
    // Side streams for independent launches (the narrowphase's per-class kernels): fork_streams()
    // makes every side stream wait for the work queued on the world's stream so far, use_stream(k)
    // sends the following launches to side stream k, join_streams() makes the world's stream wait
    // for all side streams and sends launches back to it.
    static constexpr int kSideStreams = 4;
    cudaStream_t side_[kSideStreams] = {};
    cudaEvent_t fork_ev_ = nullptr, join_ev_[kSideStreams] = {};
    cudaStream_t cur_ = nullptr;
    void fork_streams() {
        PE_CK(cudaEventRecord(fork_ev_, st_));
        for (int k = 0; k < kSideStreams; k++) PE_CK(cudaStreamWaitEvent(side_[k], fork_ev_, 0));
    }
    void use_stream(int k) { cur_ = side_[k % kSideStreams]; }
    void join_streams() {
        cur_ = nullptr;
        for (int k = 0; k < kSideStreams; k++) {
            PE_CK(cudaEventRecord(join_ev_[k], side_[k]));
            PE_CK(cudaStreamWaitEvent(st_, join_ev_[k], 0));
        }
    }
    // cooperative launch (all blocks resident; grid-wide barriers inside the kernel)
    template <class... P, class... A> void launch_coop(int id, int g, int block, void (*kern)(P...), A... args) {
        klaunch_[id]++;
        step_launches_++;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (prof_) {
            if (ev_pool_.size() < 2) { cudaEvent_t a, b; PE_CK(cudaEventCreate(&a)); PE_CK(cudaEventCreate(&b)); ev_pool_.push_back(a); ev_pool_.push_back(b); }
            e0 = ev_pool_.back(); ev_pool_.pop_back();
            e1 = ev_pool_.back(); ev_pool_.pop_back();
            PE_CK(cudaEventRecord(e0, st_));
        }
        std::tuple<P...> held(args...);   // the kernel's exact parameter types
        void* ptrs[sizeof...(P)];
        fill_ptrs(held, ptrs, std::index_sequence_for<P...>{});
        PE_CK(cudaLaunchCooperativeKernel((const void*)kern, dim3(g), dim3(block), ptrs, 0, st_));
        if (prof_) {
            PE_CK(cudaEventRecord(e1, st_));
            pending_.push_back({id, e0, e1});
        }
    }
    template <class Tup, size_t... I> static void fill_ptrs(Tup& t, void** p, std::index_sequence<I...>) {
        ((p[I] = (void*)&std::get<I>(t)), ...);
    }
    int coop_blocks_ = 0;   // co-resident blocks of k_gc_solve
    struct Pending { int id; cudaEvent_t e0, e1; };
    void resolve_prof() {
        if (pending_.empty()) return;
        PE_CK(cudaStreamSynchronize(st_));
        for (auto& q : pending_) {
            float ms = 0;
            PE_CK(cudaEventElapsedTime(&ms, q.e0, q.e1));
            kms_[q.id] += ms;
            ev_pool_.push_back(q.e0);
            ev_pool_.push_back(q.e1);
        }
        pending_.clear();
    }
    bool prof_ = false;
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> ev_pool_;
    double kms_[K_COUNT] = {};
    long long klaunch_[K_COUNT] = {};
    long long step_launches_ = 0, last_step_launches_ = 0;

    Bodies<R> bodies() {
        Bodies<R> b;
        b.f = bf_.p; b.cap = bcap_; b.n = N_; b.shape = bshape_.p; b.flags = bflags_.p; b.scene = bscene_.p;
        return b;
    }
    ShapeTable<R> shapes() const;
    // appends shapes; returns the first new index.  With `remap`, convex meshes identical to one
    // appended this way before are not appended again: remap[s] is shape s's index in the tables.
    int append_shapes(int S, const int* type, const double* param, const int* vbeg, const int* vcnt, const int* fbeg,
                      const int* fcnt, const double* hv, const int* foff, const int* fidx, std::vector<int>* remap = nullptr);
    std::unordered_map<std::string, int> hull_by_content_;
    void fill_body(R* f, size_t stride, int j, int shape, double mass, double fr, double re, double ld, double ad,
                   const double* o, const double* b, const double* v, const double* w) const;
    Results<R> results();
    Rows<R> rows();
    void scan_async(int* data, int n, int* total);   // exclusive scan in place, total to device memory
    DBuf<int> rows_total_;

    // ---- the step without host waits between its phases.  The device holds the sizes the phases
    // pass on (pairs, results, active results, island items, medium islands); kernels read them
    // there, and their grids come from upper bounds (the pair capacity), at most the GPU's resident
    // blocks.  The host waits twice per step: for the pair count (the capacities follow it) and for
    // the step's counters at its end.
    enum DevCount { DC_P = 0, DC_R, DC_A, DC_M, DC_NMED, DC_MEDCUR, DC_COUNT };
    DBuf<int> dcnt_;
    DBuf<int2> cls_rng_;   // [first, end) of each pair class in the bucketed order
    DBuf<int> cls_work_;   // per-class work cursors of the pair-at-a-time kernels
    DBuf<int> isl_med_;    // islands above small_island_items and up to big_island_items results
    const uint32_t* isl_order_ = nullptr;   // island items sorted by island (points into val_)
    // counters read back at the step's end, one copy into page-locked memory
    // (k_step_counters writes them in this order)
    enum HostStat { HS_STATUS = 0, HS_ROWS, HS_ACTIVE, HS_ISLANDS, HS_BIG, HS_COLORS, HS_P, HS_CLS, HS_COUNT = HS_CLS + PC_COUNT };
    DBuf<int> dstat_;
    int* hstat_ = nullptr;
    int h_cls_[PC_COUNT] = {};   // the last step's pair-class counts (the side-stream plan)
    int stream_of_[PC_COUNT] = {};
    void plan_streams(int* plan) const;
    int bp_count();                 // integrate's successor up to the pair count (waits for it)
    void bp_count_enqueue();        // its launches, ending with the count's copy to the host
    void run_head();                // integrate and bp_count_enqueue, replayed from a CUDA graph when enabled
    void prepare_tail(int P);       // every capacity the rest of the step needs, before any launch of it
    void bp_tail();                 // pair list, scene pair offsets, sweep axes
    void np_enqueue();              // narrowphase, no host waits
    void solve_enqueue(int mode);   // solver up to the velocity sync and the counters' copy, no host waits
    void finish(int mode);          // waits for the counters; big islands; status
    void run_tail(int mode);        // bp_tail .. solve_enqueue, replayed from a CUDA graph when enabled
    int radix_sort_dev(int bound, int key_passes, const int* nd);
    // resident blocks of a kernel at a block size and dynamic shared memory (cached), and a grid for
    // `items` items of `per_block` items per block, at most four times those (the work loops stride
    // or take items from a cursor; blocks beyond the resident ones let the block scheduler mix the
    // side streams' kernels: the batched step measured 0.12 ms faster than with resident-sized grids)
    std::map<std::tuple<const void*, int, size_t>, int> resident_;
    int sms_ = 0;
    template <class Kern> int resident(Kern kern, int block, size_t smem) {
        const auto key = std::make_tuple((const void*)kern, block, smem);
        auto it = resident_.find(key);
        if (it != resident_.end()) return it->second;
        if (sms_ == 0) PE_CK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev_));
        int b = 0;
        PE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, block, smem));
        const int r = std::max(b, 1) * sms_;
        resident_[key] = r;
        return r;
    }
    template <class Kern> int pgrid(long long items, int per_block, Kern kern, int block = kBlock, size_t smem = 0) {
        const long long g = std::max((items + per_block - 1) / per_block, 1ll);
        return (int)std::min<long long>(g, 4ll * resident(kern, block, smem));
    }
    // captured step graphs, by solver mode and contact-distance generation, with what they baked in
    struct GraphSig {
        unsigned long long gen;
        const void* order;
        int n, ns, pair_cap, rows_cap, nj, n_ign, s, side;
        int plan[PC_COUNT];
        StepParams prm;
        R margin;
        Tuning tun;
    };
    void graph_sig(GraphSig& g) const;
    cudaGraphExec_t gexec_[2][2] = {};
    GraphSig gsig_[2][2];
    GraphSig last_sig_;     // the previous step's (a capture waits for one repeat)
    cudaGraphExec_t ghead_ = nullptr;   // the head's graph (integrate and the broadphase up to the pair count)
    GraphSig gsig_head_, last_sig_head_;
    long long glaunch_head_ = 0;
    template <class F>
    void graph_run(cudaGraphExec_t& ex, GraphSig& held, long long& held_launches, GraphSig& last, const GraphSig& sig, F&& enqueue);
    long long glaunch_[2][2] = {};
    bool graphs_ = true, capturing_ = false;
    long long steps_since_plan_ = 0;
    R* staging(size_t n);         // pinned host buffer of at least n reals
    R* stage_ = nullptr;
    size_t stage_n_ = 0;
    void radix_sort(int n, int n_scene_passes);
    int radix_sort_keys(int n, int key_passes, int scene_passes);   // returns the buffer holding the result
    void ensure_pair_capacity(int P);
    void ev_begin(int phase);
    void ev_end(int phase);
    void ev_collect();
    int grid(int n) const { return (n + kBlock - 1) / kBlock; }
    int grid_warps(int n) const { return (int)(((size_t)n * 32 + kBlock - 1) / kBlock); }   // one warp per item

    int dev_;
    cudaStream_t st_ = nullptr;
    cudaEvent_t ev_[5][2];
    bool ev_open_[5] = {false, false, false, false, false};
    double ms_[5] = {0, 0, 0, 0, 0};
    StepParams prm_{0.01, {0, -9.8, 0}, 10};
    R margin_ = 0;   // contact margin of the pair algorithms (PE_MARGIN, phys_general.h:45)
    Tuning tun_;     // scheduling settings
    // shapes
    int S_ = 0;
    DBuf<int> stype_, shull_, hvbeg_, hvcnt_, hfbeg_, hfcnt_, hebeg_, hecnt_, hfoff_, hfidx_;
    DBuf<R> sparam_, hv_, hfn_, hfmin_, hfmax_, hea_, heb_, hed_, hrad_;
    std::vector<int> h_stype_;
    std::vector<R> h_sparam_;
    std::vector<M3<R>> h_sinertia_;
    // host copies of the shape tables (shapes are only ever appended after set_shapes)
    std::vector<int> h_shull_, h_hvb_, h_hvc_, h_hfb_, h_hfc_, h_heb_, h_hec_, h_foff_, h_fidx_;
    std::vector<R> h_hv_, h_fn_, h_fmn_, h_fmx_, h_ea_, h_eb_, h_hrad_;   // h_hrad_: inner, outer radius per hull
    // concave meshes' face-tree leaves (per hull: first leaf and count; per leaf: face range and box)
    DBuf<int> hlbeg_, hlcnt_, lfbeg_, lfcnt_;
    DBuf<R> lfmin_, lfmax_;
    std::vector<int> h_hlb_, h_hlc_, h_lfb_, h_lfc_;
    std::vector<R> h_lfmn_, h_lfmx_;
    // compound children (per shape: first child and count; per child: shape and 12-real transform)
    DBuf<int> cbeg_, ccnt_, cshape_;
    DBuf<R> cxf_;
    std::vector<int> h_cbeg_, h_ccnt_, h_cshape_;
    std::vector<char> h_cready_;
    std::vector<R> h_cxf_;
    // joints (World::_constraints) and ignored collision pairs
    int n_joints_ = 0, n_ign_ = 0;
    DBuf<int> jtype_, jflag_, ign_off_, ign_ids_;
    DBuf<int2> jbody_;
    DBuf<R> jparam_, jrow_;
    Joints<R> joints() {
        Joints<R> j;
        j.n = n_joints_; j.type = jtype_.p; j.body = jbody_.p; j.flag = jflag_.p; j.param = jparam_.p; j.row = jrow_.p;
        return j;
    }
    // bodies
    int N_ = 0, bcap_ = 0;
    DBuf<R> bf_;
    DBuf<int> bshape_, bflags_, bscene_;
    // scenes
    int NS_ = 1;
    std::vector<int> h_scene_off_;
    DBuf<int> scene_off_, scene_axis_, pair_scene_off_, res_scene_off_, prev_res_off_;
    // broadphase
    DBuf<uint64_t> key_[2];
    DBuf<uint32_t> key2_[2], val_[2];
    DBuf<int> hist_, aux_, total_, count_, status_;
    DBuf<R> smn_, smx_;
    DBuf<int> sflag_, ssc_, bp_stage_, bp_big_, bp_nbig_;
    DBuf<int> bp_wend_, bp_csize_, bp_nch_, bp_choff_, bp_ctot_, bp_ccount_, bp_cpref_;   // crowded windows in chunks
    static constexpr int kBigSweepBlocks = 152;   // blocks that share the crowded positions
    uint32_t* order_ = nullptr;   // sorted body order (points into val_)
    int max_scene_ = 0;           // bodies of the largest scene (the crowded-window kernels run above kBigWindow)
    DBuf<int2> pairs_;
    int P_ = 0, pair_cap_ = 0;
    // narrowphase
    DBuf<int> cls_, cls_count_, order_np_;
    DBuf<int> res_a_, res_b_, res_np_;
    DBuf<R> res_fr_, res_re_, res_pts_, res_dist_[2], sat_out_;
    int cur_dist_ = 0;
    int R_ = 0;
    std::vector<int> h_pair_scene_off_;
    // solver
    DBuf<int> row_off_, active_, color_, claim_, parent_, isl_flag_, isl_off_, isl_n_, ncol_;
    DBuf<uint32_t> isl_corder_;
    DBuf<int> gc_big_, gc_n_, gc_cnt_, gc_cursor_, gc_cstart_, gc_ccount_;
    DBuf<unsigned long long> gc_mask_, gc_claim_;
    DBuf<double> xfer_;   // state transfers in the C ABI's layout
    DBuf<int> gc_left_;   // items left after each colouring round
    DBuf<int> gc_level_;  // coloured mode: exact levels of a big island beside its first-fit colours
    void solve_big_islands(int nb, const uint32_t* order, bool exact);
    DBuf<R> rows_;
    int rows_cap_ = 0, n_rows_ = 0, n_active_ = 0, n_colors_ = 0, n_islands_ = 0;
    bool sat_attr_ = false;
};

} // namespace pe
