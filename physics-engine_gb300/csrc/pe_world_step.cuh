// World<R> member definitions, part 2: the step, phase by phase (sort and scan utilities,
// integrate, broadphase, narrowphase, solve, big islands), and its captured CUDA graph.
#pragma once
#include "pe_world_setup.cuh"

namespace pe {

// ------------------------------------------------------------------ utilities
template <class R> void World<R>::scan_async(int* data, int n, int* total) {
    const int tiles = (n + 1023) / 1024;
    if (tiles <= kSmallScanTiles) {
        launch(K_SCAN, 1, k_scan_aux, data, n, total);
    } else {
        aux_.ensure(tiles + 1);
        launch(K_SCAN, tiles, k_scan_tiles, data, n, aux_.p);
        launch(K_SCAN, 1, k_scan_aux, aux_.p, tiles, total);
        launch(K_SCAN, tiles, k_scan_add, data, n, aux_.p);
    }
}

template <class R> void World<R>::radix_sort(int n, int scene_passes) {
    order_ = val_[radix_sort_keys(n, (int)sizeof(R), scene_passes)].p;
}

template <class R> int World<R>::radix_sort_keys(int n, int key_passes, int scene_passes) {
    if (scene_passes == 0 && n <= kSceneSortMax) {   // small: one block, one launch
        launch_block(K_RADIX, 1, kSceneSortBlock, k_sort_pairs_block, (const uint64_t*)key_[0].p, (const uint32_t*)val_[0].p, n,
                     (const int*)nullptr, key_[1].p, val_[1].p);
        return 1;
    }
    const int tiles = (n + kRadixTile - 1) / kRadixTile;
    hist_.ensure((size_t)256 * tiles + 1);
    aux_.ensure((256 * tiles + 1023) / 1024 + 1);
    int cur = 0;
    auto pass = [&](int shift, int use2) {
        launch(K_RADIX, tiles, k_radix_hist, (const uint64_t*)key_[cur].p, (const uint32_t*)key2_[cur].p, n, (const int*)nullptr, -1, shift,
               use2, hist_.p, tiles);
        scan_async(hist_.p, 256 * tiles, total_.p);
        launch(K_RADIX, tiles, k_radix_scatter, (const uint64_t*)key_[cur].p, (const uint32_t*)key2_[cur].p, (const uint32_t*)val_[cur].p,
               key_[cur ^ 1].p, key2_[cur ^ 1].p, val_[cur ^ 1].p, n, (const int*)nullptr, -1, shift, use2, (const int*)hist_.p, tiles);
        cur ^= 1;
    };
    for (int s = 0; s < key_passes * 8; s += 8) pass(s, 0);
    for (int s = 0; s < scene_passes * 8; s += 8) pass(s, 1);
    return cur;
}

// Sort of up to `bound` keys whose count is on the device (*nd): one block when it is at most
// kSceneSortMax, the radix passes above (each launch does nothing for the other case).  Both end
// in the buffer returned.
template <class R> int World<R>::radix_sort_dev(int bound, int key_passes, const int* nd) {
    if (bound <= kSceneSortMax) {
        launch_block(K_RADIX, 1, kSceneSortBlock, k_sort_pairs_block, (const uint64_t*)key_[0].p, (const uint32_t*)val_[0].p, bound, nd,
                     key_[1].p, val_[1].p);
        return 1;
    }
    const int fin = key_passes & 1;   // the buffer the passes end in (the block sort may write its input)
    launch_block(K_RADIX, 1, kSceneSortBlock, k_sort_pairs_block, (const uint64_t*)key_[0].p, (const uint32_t*)val_[0].p, bound, nd,
                 key_[fin].p, val_[fin].p);
    const int tiles = (bound + kRadixTile - 1) / kRadixTile;
    int cur = 0;
    for (int s = 0; s < key_passes * 8; s += 8) {
        launch(K_RADIX, tiles, k_radix_hist, (const uint64_t*)key_[cur].p, (const uint32_t*)key2_[cur].p, bound, nd, kSceneSortMax, s, 0,
               hist_.p, tiles);
        scan_async(hist_.p, 256 * tiles, total_.p);
        launch(K_RADIX, tiles, k_radix_scatter, (const uint64_t*)key_[cur].p, (const uint32_t*)key2_[cur].p, (const uint32_t*)val_[cur].p,
               key_[cur ^ 1].p, key2_[cur ^ 1].p, val_[cur ^ 1].p, bound, nd, kSceneSortMax, s, 0, (const int*)hist_.p, tiles);
        cur ^= 1;
    }
    return fin;
}

template <class R> void World<R>::ensure_pair_capacity(int P) {
    if (P <= pair_cap_) return;
    const int cap = std::max(P + P / 2, 1024);
    pairs_.ensure(cap);
    cls_.ensure(cap); order_np_.ensure(cap);
    res_a_.ensure(cap); res_b_.ensure(cap); res_np_.ensure(cap + 1);
    res_fr_.ensure(cap); res_re_.ensure(cap);
    res_pts_.ensure((size_t)NPF * cap * kSlots);
    // result slot distances survive between steps: grow both generations keeping contents
    res_dist_[0].ensure((size_t)cap * kSlots, true);
    res_dist_[1].ensure((size_t)cap * kSlots, true);
    row_off_.ensure(cap + 1); active_.ensure(cap + 1); color_.ensure(cap + 1);
    sat_out_.ensure((size_t)cap * kSatOut);
    // point buffer: field-major over the capacity; its contents live for one step only
    pair_cap_ = cap;
}

// ------------------------------------------------------------------ phases
template <class R> void World<R>::integrate() {
    if (N_ == 0) return;
    launch(K_INTEGRATE, grid(N_), k_integrate<R>, bodies(), shapes(), prm_, 1);
    PE_CK(cudaGetLastError());
}

// Broadphase up to the pair count: sort, sweep counts, scan; the host waits for the count (the
// pair capacity follows it).  The count also stays on the device for the kernels after it.
template <class R> int World<R>::bp_count() {
    if (N_ < 2) return P_;   // the reference leaves the pair list untouched below two bodies
    bp_count_enqueue();
    PE_CK(cudaStreamSynchronize(st_));
    return hstat_[HS_P];
}

// the launches of bp_count, ending with the count's copy into page-locked memory (no wait)
template <class R> void World<R>::bp_count_enqueue() {
    const int n = N_;
    if (n < 2) return;
    for (int k = 0; k < 2; k++) { key_[k].ensure(n); key2_[k].ensure(n); val_[k].ensure(n); }
    smn_.ensure((size_t)3 * n); smx_.ensure((size_t)3 * n); sflag_.ensure(n); ssc_.ensure(n);
    count_.ensure(n + 1);
    max_scene_ = 0;
    for (int s = 0; s < NS_; s++) max_scene_ = std::max(max_scene_, h_scene_off_[s + 1] - h_scene_off_[s]);
    if (max_scene_ <= std::min(tun_.scene_sort_max, kSceneSortMax)) {   // every scene sorted inside one block
        launch_block(K_RADIX, NS_, kSceneSortBlock, k_bp_sort_scenes<R>, bodies(), (const int*)scene_axis_.p, (const int*)scene_off_.p,
                     val_[0].p);
        order_ = val_[0].p;
    } else {
        launch(K_BP_KEYS, grid(n), k_bp_keys<R>, bodies(), scene_axis_.p, key_[0].p, key2_[0].p, val_[0].p);
        int scene_passes = 0;
        for (int m = NS_ - 1; m > 0; m >>= 8) scene_passes++;
        radix_sort(n, scene_passes);
    }
    launch(K_BP_GATHER, grid(n), k_bp_gather<R>, bodies(), order_, smn_.p, smx_.p, sflag_.p, ssc_.p);
    bp_stage_.ensure((size_t)n * kStage);
    bp_big_.ensure(n + 1);
    bp_nbig_.ensure(1);
    PE_CK(cudaMemsetAsync(bp_nbig_.p, 0, sizeof(int), st_));
    IgnoreLists ign;
    if (n_ign_ > 0) { ign.off = ign_off_.p; ign.ids = ign_ids_.p; ign.order = order_; }
    launch(K_BP_SWEEP, grid_warps(n), k_bp_count<R>, n, scene_axis_.p, smn_.p, smx_.p, sflag_.p, ssc_.p, count_.p, bp_stage_.p,
           bp_big_.p, bp_nbig_.p, ign);
    // crowded positions: windows in chunks of one block each (at most kMaxChunks per position); a
    // window holds at most the scene's other bodies, so scenes of at most kBigWindow bodies have none
    const bool crowded = max_scene_ > kBigWindow;
    bp_wend_.ensure(n + 1); bp_csize_.ensure(n + 1); bp_nch_.ensure(n + 1); bp_choff_.ensure(n + 1); bp_ctot_.ensure(1);
    bp_ccount_.ensure((size_t)kMaxChunks * n + 1); bp_cpref_.ensure((size_t)kMaxChunks * n + 1);
    if (crowded) launch(K_BP_SWEEP, kBigSweepBlocks, k_bp_big_windows<R>, n, (const int*)scene_axis_.p, (const int*)scene_off_.p, (const R*)smn_.p,
           (const R*)smx_.p, (const int*)ssc_.p, (const int*)bp_big_.p, (const int*)bp_nbig_.p, bp_wend_.p, bp_csize_.p, bp_nch_.p);
    if (crowded) launch_block(K_BP_SWEEP, 1, 32, k_bp_chunk_offsets, (const int*)bp_nbig_.p, (const int*)bp_nch_.p, bp_choff_.p, bp_ctot_.p);
    if (crowded) launch(K_BP_SWEEP, 2 * kBigSweepBlocks, k_bp_count_chunks<R>, n, (const R*)smn_.p, (const R*)smx_.p, (const int*)sflag_.p,
           (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_wend_.p, (const int*)bp_csize_.p, (const int*)bp_choff_.p,
           (const int*)bp_ctot_.p, bp_ccount_.p, ign);
    if (crowded) launch(K_BP_SWEEP, kBigSweepBlocks, k_bp_chunk_sums, (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_choff_.p,
           (const int*)bp_nch_.p, (const int*)bp_ccount_.p, bp_cpref_.p, count_.p);
    PE_CK(cudaMemsetAsync(count_.p + n, 0, sizeof(int), st_));
    aux_.ensure((n + 1 + 1023) / 1024 + 1);
    scan_async(count_.p, n + 1, dcnt_.p + DC_P);
    PE_CK(cudaMemcpyAsync(hstat_ + HS_P, dcnt_.p + DC_P, sizeof(int), cudaMemcpyDeviceToHost, st_));
}

// Every buffer the rest of the step writes, sized for P pairs before any of its launches, so that
// nothing is allocated while a step graph is captured.  Island items (active results and joints)
// are bounded by the pair capacity plus the joints.
template <class R> void World<R>::prepare_tail(int P) {
    ensure_pair_capacity(std::max(P, 1));
    // a result has at most kSlots points, so kSlots rows per pair slot always fit
    if ((long long)kSlots * pair_cap_ > rows_cap_) {
        rows_cap_ = kSlots * pair_cap_ + kSlots * pair_cap_ / 4;
        rows_.ensure((size_t)NRF * rows_cap_);
    }
    const int bound = pair_cap_ + n_joints_;
    const int keys = std::max(N_, bound);
    // the sort buffers also hold the broadphase's body order until the pair list is written: a
    // growth keeps their contents and order_ follows its buffer
    const int oi = order_ == val_[1].p ? 1 : 0;
    const bool ordered = order_ != nullptr;
    for (int k = 0; k < 2; k++) { key_[k].ensure(keys); key2_[k].ensure(keys); val_[k].ensure(keys, true); }
    if (ordered) order_ = val_[oi].p;
    const int tiles = (bound + kRadixTile - 1) / kRadixTile;
    hist_.ensure((size_t)256 * tiles + 1);
    aux_.ensure(std::max((256 * tiles + 1023) / 1024, (std::max(bound, N_) + 1 + 1023) / 1024) + 1);
    isl_flag_.ensure(bound + 1); isl_off_.ensure(bound + 1); isl_med_.ensure(bound + 1); gc_big_.ensure(bound + 1);
    isl_corder_.ensure(bound); color_.ensure(bound + 1);
    isl_n_.ensure(1); ncol_.ensure(1); gc_n_.ensure(2);
    parent_.ensure(N_ + 1);
    cls_count_.ensure(2 * PC_COUNT); cls_rng_.ensure(PC_COUNT); cls_work_.ensure(PC_COUNT);
    if (!sat_attr_) {   // dynamic shared memory of the staged SAT kernels (above the 48 KB default for FP64)
        const int light = (int)(kSatWarps * sat_group_reals<R>(1) * sizeof(R));
        PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_BOX, ST_HULL>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
        PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_HULL, ST_BOX>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
        PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_HULL, ST_HULL>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
        PE_CK(cudaFuncSetAttribute(k_np_sat<R, 1, ST_CYLINDER, ST_CYLINDER>, cudaFuncAttributeMaxDynamicSharedMemorySize, light));
        PE_CK(cudaFuncSetAttribute(k_np_sat<R, kSatGroup, -1, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sat_group_reals<R>(kSatGroup) * sizeof(R))));
        sat_attr_ = true;
    }
}

// the pair list from the counted sweep, each scene's first pair, and the scenes' next sweep axes
template <class R> void World<R>::bp_tail() {
    const int n = N_;
    if (n < 2) return;
    IgnoreLists ign;
    if (n_ign_ > 0) { ign.off = ign_off_.p; ign.ids = ign_ids_.p; ign.order = order_; }
    launch(K_BP_SWEEP, grid_warps(n), k_bp_write<R>, n, scene_axis_.p, smn_.p, smx_.p, sflag_.p, ssc_.p, order_, count_.p, bp_stage_.p,
           pairs_.p, pair_cap_, status_.p, ign);
    if (max_scene_ > kBigWindow)
        launch(K_BP_SWEEP, 2 * kBigSweepBlocks, k_bp_write_chunks<R>, n, (const R*)smn_.p, (const R*)smx_.p, (const int*)sflag_.p,
               (const uint32_t*)order_, (const int*)count_.p, (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_wend_.p,
               (const int*)bp_csize_.p, (const int*)bp_choff_.p, (const int*)bp_ctot_.p, (const int*)bp_cpref_.p, pairs_.p, pair_cap_,
               status_.p, ign);
    launch(K_MISC, grid(NS_ + 1), k_scene_pair_off, NS_, scene_off_.p, count_.p, n, pair_scene_off_.p);
    launch_block(K_BP_AXIS, NS_, 64, k_bp_axis<R>, (const R*)smn_.p, (const R*)smx_.p, n, (const int*)scene_off_.p, scene_axis_.p);
}

template <class R> int World<R>::broadphase() {
    const int P = bp_count();
    prepare_tail(P);
    bp_tail();
    PE_CK(cudaGetLastError());
    P_ = P;
    return P;
}

// Side streams for the pair classes, largest estimated work first (the last counts x a rough
// per-pair cost), each to the least loaded stream.
template <class R> void World<R>::plan_streams(int* plan) const {
    static_assert(PC_COUNT == 15, "one cost per pair class");
    static constexpr double kClassCost[PC_COUNT] = {2, 1, 1, 1, 4, 20, 6, 12, 400, 40, 40, 60, 20, 30, 30};
    int order_c[PC_COUNT];
    double load[kSideStreams] = {};
    for (int c = 0; c < PC_COUNT; c++) order_c[c] = c;
    std::stable_sort(order_c, order_c + PC_COUNT, [&](int a, int b) { return h_cls_[a] * kClassCost[a] > h_cls_[b] * kClassCost[b]; });
    for (int k = 0; k < PC_COUNT; k++) {
        const int c = order_c[k];
        const int best = (int)(std::min_element(load, load + kSideStreams) - load);
        plan[c] = best;
        load[best] += h_cls_[c] * kClassCost[c];
    }
}

// Narrowphase without host waits: pairs classified and bucketed by class on the device, the class
// ranges computed there, and every class's kernel launched over its range (grids from the pair
// capacity, persistent up to the resident blocks), side by side on the side streams.
template <class R> void World<R>::np_enqueue() {
    // the results of the previous step become the pool the new step draws stale slots from
    PE_CK(cudaMemcpyAsync(prev_res_off_.p, res_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    const int cap = pair_cap_;
    const int* Pd = dcnt_.p + DC_P;
    const Results<R> rs = results();
    const Bodies<R> bd = bodies();
    const ShapeTable<R> sh = shapes();
    PE_CK(cudaMemsetAsync(cls_count_.p, 0, PC_COUNT * sizeof(int), st_));
    launch(K_NP_BUCKET, pgrid(cap, kBlock, k_np_classify<R>), k_np_classify<R>, Pd, (const int2*)pairs_.p, bd, sh, cls_.p, cls_count_.p,
           (long long)tun_.sat_heavy_cost);
    launch_block(K_NP_BUCKET, 1, 32, k_np_ranges, (const int*)cls_count_.p, cls_count_.p + PC_COUNT, cls_rng_.p, cls_work_.p);
    launch(K_NP_BUCKET, pgrid(cap, kBlock, k_np_bucket), k_np_bucket, Pd, (const int*)cls_.p, cls_count_.p + PC_COUNT, order_np_.p);
    // The classes' kernels touch disjoint pairs and results: they run side by side on the side
    // streams, so the long tails of the per-pair kernels overlap the other classes.
    fork_streams();
    for (int c = 0; c < PC_COUNT; c++) {
        use_stream(stream_of_[c] % tun_.side_streams);
        const int2* rg = cls_rng_.p + c;
        int* wk = cls_work_.p + c;
        const int* on = order_np_.p;
        const int2* pp = pairs_.p;
        const int* pso = pair_scene_off_.p;
        const int* pro = prev_res_off_.p;
        switch (c) {
            case PC_BOX_BOX: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_BOX_BOX>), k_np_class<R, PC_BOX_BOX>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_BOX_SPHERE: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_BOX_SPHERE>), k_np_class<R, PC_BOX_SPHERE>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_SPHERE_SPHERE: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_SPHERE_SPHERE>), k_np_class<R, PC_SPHERE_SPHERE>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_SPHERE_CYL: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_SPHERE_CYL>), k_np_class<R, PC_SPHERE_CYL>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_BOX_CYL: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_BOX_CYL>), k_np_class<R, PC_BOX_CYL>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_CONCAVE: launch(K_NP, pgrid(cap, kBlock, k_np_class<R, PC_CONCAVE>), k_np_class<R, PC_CONCAVE>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_COMPOUND: launch(K_NP, pgrid(cap, kBlock, k_np_compound<R>), k_np_compound<R>, rg, on, pp, bd, sh, rs, pso, pro); break;
            case PC_SPHERE_HULL: {
                const int w = sphere_hull_warps<R>();
                launch_block(K_NP, pgrid(cap, w, k_np_sphere_hull<R>, 32 * w), 32 * w, k_np_sphere_hull<R>, rg, wk, on, pp, bd, sh, rs, pso, pro);
                break;
            }
            case PC_CYL_HULL: {
                const int w = cyl_hull_warps<R>();
                launch_block(K_NP, pgrid(cap, w, k_np_cyl_hull<R>, 32 * w), 32 * w, k_np_cyl_hull<R>, rg, wk, on, pp, bd, sh, rs, pso, pro);
                break;
            }
            case PC_CONVEX:
            case PC_CONVEX_HULL_BOX:
            case PC_CONVEX_HULL_HULL:
            case PC_CONVEX_CYL_CYL: {
                const size_t smem = (size_t)kSatWarps * sat_group_reals<R>(1) * sizeof(R);
                const int bs = 32 * kSatWarps;
                auto kern = c == PC_CONVEX ? k_np_sat<R, 1, ST_BOX, ST_HULL>
                          : c == PC_CONVEX_HULL_BOX ? k_np_sat<R, 1, ST_HULL, ST_BOX>
                          : c == PC_CONVEX_HULL_HULL ? k_np_sat<R, 1, ST_HULL, ST_HULL>
                          : k_np_sat<R, 1, ST_CYLINDER, ST_CYLINDER>;
                launch_smem(K_NP_SAT, pgrid(cap, kSatWarps, kern, bs, smem), bs, smem, kern, rg, wk, on, pp, bd, sh, sat_out_.p);
                launch(K_NP_SAT, pgrid(cap, kBlock, k_np_sat_finish<R>), k_np_sat_finish<R>, rg, on, pp, bd, sh, rs, pso, pro,
                       (const R*)sat_out_.p);
                break;
            }
            case PC_CONVEX_HEAVY: {
                const size_t smem = (size_t)sat_group_reals<R>(kSatGroup) * sizeof(R);
                auto kern = k_np_sat<R, kSatGroup, -1, -1>;
                launch_smem(K_NP_SAT, pgrid(cap, 1, kern, 32 * kSatGroup, smem), 32 * kSatGroup, smem, kern, rg, wk, on, pp, bd, sh, sat_out_.p);
                launch(K_NP_SAT, pgrid(cap, kBlock, k_np_sat_finish<R>), k_np_sat_finish<R>, rg, on, pp, bd, sh, rs, pso, pro,
                       (const R*)sat_out_.p);
                break;
            }
            default:   // PC_CONVEX_BIG
                launch(K_NP_SAT, pgrid(cap, kBlock / 32, k_np_sat_big<R>), k_np_sat_big<R>, rg, wk, on, pp, bd, sh, rs, pso, pro);
                break;
        }
    }
    join_streams();
    PE_CK(cudaMemcpyAsync(res_scene_off_.p, pair_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    PE_CK(cudaMemcpyAsync(dcnt_.p + DC_R, dcnt_.p + DC_P, sizeof(int), cudaMemcpyDeviceToDevice, st_));
}

template <class R> void World<R>::narrowphase() {
    prepare_tail(P_);
    plan_streams(stream_of_);
    cur_dist_ ^= 1;
    np_enqueue();
    PE_CK(cudaGetLastError());
    R_ = P_;
}

// Solver without host waits, up to the velocity sync: rows, active results, islands (union-find,
// sort by island, offsets), the small islands one thread each, the medium ones a block each (exact
// levels in serial-order mode, colours in coloured mode), the big islands listed for finish(); then
// the step's counters are copied to the host in one transfer.
template <class R> void World<R>::solve_enqueue(int mode) {
    if (N_ == 0) return;
    const int cap = pair_cap_, NJ = n_joints_, bound = cap + NJ;
    const int* Rd = dcnt_.p + DC_R;
    launch(K_SI_MISC, grid(N_), k_si_clear<R>, bodies());
    // rows: one per contact point, results' rows contiguous in result order
    launch(K_SI_MISC, pgrid(cap + 1, kBlock, k_rows_init), k_rows_init, Rd, cap, (const int*)res_np_.p, row_off_.p);
    scan_async(row_off_.p, cap + 1, rows_total_.p);
    launch(K_SI_SETUP, pgrid(cap, kBlock, k_si_setup<R>), k_si_setup<R>, Rd, results(), bodies(), rows(), (const int*)row_off_.p, prm_,
           status_.p);
    // results with points, in result order
    launch(K_SI_MISC, pgrid(cap + 1, kBlock, k_active_flags), k_active_flags, Rd, cap, (const int*)res_np_.p, color_.p);
    scan_async(color_.p, cap + 1, dcnt_.p + DC_A);
    launch(K_SI_MISC, pgrid(cap, kBlock, k_active_compact), k_active_compact, Rd, (const int*)res_np_.p, (const int*)color_.p, active_.p);
    const Joints<R> jt = joints();
    if (NJ > 0) launch(K_SI_SETUP, grid(NJ), k_joint_init<R>, jt, bodies(), prm_);
    // islands: union-find over dynamic bodies linked by contacts and joints; items (active results
    // in result order, then joints in order) sorted by island label, stably
    const int* Ad = dcnt_.p + DC_A;
    int* Md = dcnt_.p + DC_M;
    launch_block(K_ISLAND, 1, 32, k_count_add, Ad, NJ, Md);
    launch(K_ISLAND, grid(N_), k_isl_init, N_, parent_.p);
    launch(K_ISLAND, pgrid(cap, kBlock, k_isl_union<R>), k_isl_union<R>, Ad, (const int*)active_.p, results(), bodies(), parent_.p);
    if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_union_joints<R>, jt, bodies(), parent_.p);
    launch(K_ISLAND, pgrid(cap, kBlock, k_isl_keys<R>), k_isl_keys<R>, Ad, (const int*)active_.p, results(), bodies(), (const int*)parent_.p,
           key_[0].p, key2_[0].p, val_[0].p);
    if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_keys_joints<R>, jt, bodies(), (const int*)parent_.p, Ad, key_[0].p, key2_[0].p, val_[0].p);
    int label_passes = 0;
    for (int m = NJ > 0 ? N_ : N_ - 1; m > 0; m >>= 8) label_passes++;   // joint labels reach n_bodies
    const int cur = radix_sort_dev(bound, label_passes, Md);
    const uint64_t* skey = key_[cur].p;
    const uint32_t* order = val_[cur].p;
    isl_order_ = order;
    launch(K_ISLAND, pgrid(bound + 1, kBlock, k_isl_flags), k_isl_flags, (const int*)Md, bound, skey, isl_flag_.p);
    scan_async(isl_flag_.p, bound + 1, isl_n_.p);
    launch(K_ISLAND, pgrid(bound + 1, kBlock, k_isl_offsets), k_isl_offsets, (const int*)Md, skey, (const int*)isl_flag_.p, isl_off_.p,
           isl_n_.p);
    const int small = tun_.small_island_items, big = tun_.big_island_items;
    // islands of up to small_island_items items: one thread each
    launch(K_SI_SERIAL, pgrid(bound, kBlock, k_isl_serial<R>), k_isl_serial<R>, (const int*)isl_n_.p, (const int*)isl_off_.p, order,
           results(), jt, bodies(), rows(), (const int*)row_off_.p, prm_.iterations, small);
    // islands of small_island_items + 1 .. big_island_items items: listed, then a block each
    PE_CK(cudaMemsetAsync(dcnt_.p + DC_NMED, 0, 2 * sizeof(int), st_));
    launch(K_ISLAND, pgrid(bound, kBlock, k_isl_pick), k_isl_pick, (const int*)isl_n_.p, (const int*)isl_off_.p, small, big, isl_med_.p,
           dcnt_.p + DC_NMED);
    const long long med = (long long)bound / (small + 1) + 1;   // at most this many such islands
    if (mode == 0) {
        // serial order: the exact level schedule
        const int g = (int)std::min<long long>(med, resident(k_isl_levels<R>, tun_.level_block, 0));
        launch_block(K_SI_SERIAL, g, tun_.level_block, k_isl_levels<R>, (const int*)isl_med_.p, (const int*)(dcnt_.p + DC_NMED),
                     dcnt_.p + DC_MEDCUR, (const int*)isl_off_.p, order, results(), jt, bodies(), rows(), (const int*)row_off_.p,
                     prm_.iterations, small, big, claim_.p, color_.p, isl_corder_.p);
    } else {
        PE_CK(cudaMemsetAsync(ncol_.p, 0, sizeof(int), st_));
        const int g = (int)std::min<long long>(med, resident(k_isl_colored<R>, tun_.color_block, 0));
        launch_block(K_SI_COLOR, g, tun_.color_block, k_isl_colored<R>, (const int*)isl_med_.p, (const int*)(dcnt_.p + DC_NMED),
                     dcnt_.p + DC_MEDCUR, (const int*)isl_off_.p, order, results(), jt, bodies(), rows(), (const int*)row_off_.p,
                     prm_.iterations, small, big, claim_.p, color_.p, isl_corder_.p, ncol_.p);
    }
    // islands above big_island_items: listed here, solved by finish() after the counters are read
    PE_CK(cudaMemsetAsync(gc_n_.p, 0, sizeof(int), st_));
    launch(K_SI_COLOR, pgrid(bound, kBlock, k_isl_big), k_isl_big, (const int*)isl_n_.p, (const int*)isl_off_.p, gc_big_.p, gc_n_.p, big);
    launch(K_SI_MISC, grid(N_), k_si_sync<R>, bodies());
    launch_block(K_MISC, 1, 32, k_step_counters, (const int*)status_.p, (const int*)rows_total_.p, Ad, (const int*)isl_n_.p,
                 (const int*)gc_n_.p, mode == 0 ? (const int*)nullptr : (const int*)ncol_.p, (const int*)cls_count_.p, dstat_.p);
    PE_CK(cudaMemcpyAsync(hstat_, dstat_.p, HS_COUNT * sizeof(int), cudaMemcpyDeviceToHost, st_));
}

// The step's second host wait: its counters; then the big islands (host-driven, rare), whose
// solve ends with a second velocity sync; then the status.
template <class R> void World<R>::finish(int mode) {
    PE_CK(cudaStreamSynchronize(st_));
    if (N_ == 0) return;
    n_rows_ = hstat_[HS_ROWS];
    n_active_ = hstat_[HS_ACTIVE];
    n_islands_ = hstat_[HS_ISLANDS];
    n_colors_ = mode == 0 ? 0 : hstat_[HS_COLORS];
    for (int c = 0; c < PC_COUNT; c++) h_cls_[c] = hstat_[HS_CLS + c];
    const int status = hstat_[HS_STATUS], nb = hstat_[HS_BIG];
    if (status) {
        PE_CK(cudaMemsetAsync(status_.p, 0, sizeof(int), st_));
        PE_CK(cudaStreamSynchronize(st_));
        throw std::runtime_error("device capacity overflow (status " + std::to_string(status) + ")");
    }
    if (nb > 0) {
        solve_big_islands(nb, isl_order_, mode == 0);
        launch(K_SI_MISC, grid(N_), k_si_sync<R>, bodies());
        ev_end(3);   // the solve and the step end after the big islands
        ev_end(4);
        PE_CK(cudaGetLastError());
    }
}

template <class R> void World<R>::solve(int mode) {
    prepare_tail(R_);
    solve_enqueue(mode);
    PE_CK(cudaGetLastError());
    finish(mode);
}

// the nb islands above big_island_items results (listed in gc_big_): grid-wide colouring rounds,
// then one launch per colour and iteration (see k_gc_*)
template <class R> void World<R>::solve_big_islands(int nb, const uint32_t* order, bool exact) {
    std::vector<int> big(nb);
    PE_CK(cudaMemcpy(big.data(), gc_big_.p, nb * sizeof(int), cudaMemcpyDeviceToHost));
    std::sort(big.begin(), big.end());
    gc_cnt_.ensure(kMaxColorsBig + 1);
    gc_cursor_.ensure(kMaxColorsBig);
    const Results<R> rs = results();
    const Joints<R> jt = joints();
    const Bodies<R> bd = bodies();
    const Rows<R> rw = rows();
    std::vector<int> cnt(kMaxColorsBig + 1), start(kMaxColorsBig), cur(kMaxColorsBig);
    for (int s : big) {
        int lh[2];
        PE_CK(cudaMemcpy(lh, isl_off_.p + s, 2 * sizeof(int), cudaMemcpyDeviceToHost));
        const int lo = lh[0], m = lh[1] - lh[0], g = grid(m);
        PE_CK(cudaMemsetAsync(color_.p + lo, 0xff, (size_t)m * sizeof(int), st_));   // -1: uncoloured
        unsigned long long* mask = nullptr;   // exact level schedule: colour = round
        if (!exact) {
            gc_mask_.ensure(N_ + 1);
            mask = gc_mask_.p;
            launch(K_GC_COLOR, g, k_gc_mask_reset<R>, lo, m, order, rs, jt, mask);
        }
        // colouring rounds, the remaining count read back every 8 rounds (extra rounds find nothing to do)
        // all rounds in one cooperative launch (up to kMaxColorsBig - 1; items left over take the last colour)
        if (coop_blocks_ == 0) {
            int per_sm = 0, sms = 0;
            PE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gc_solve<R>, kBlock, 0));
            int per_sm2 = 0;
            PE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_gc_rounds<R>, kBlock, 0));
            PE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_));
            coop_blocks_ = std::max(std::min(per_sm, per_sm2), 1) * sms;
        }
        gc_left_.ensure(kMaxColorsBig);
        PE_CK(cudaMemsetAsync(gc_left_.p, 0, kMaxColorsBig * sizeof(int), st_));
        gc_claim_.ensure(N_ + 1);
        int* level = nullptr;   // coloured mode: the exact levels beside the first-fit colours
        if (!exact) {
            gc_level_.ensure((size_t)(lo + m));
            level = gc_level_.p;
            PE_CK(cudaMemsetAsync(level + lo, 0xff, (size_t)m * sizeof(int), st_));
        }
        launch_coop(K_GC_COLOR, coop_blocks_, kBlock, k_gc_rounds<R>, lo, m, order, rs, jt, bd, gc_claim_.p, color_.p, mask, gc_left_.p,
                    kMaxColorsBig - 1, gc_n_.p + 1, level);
        int ncol = 0;
        PE_CK(cudaMemcpyAsync(&ncol, gc_n_.p + 1, sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaStreamSynchronize(st_));
        // Coloured mode keeps the exact levels (the reference's order, as in serial-order mode) when
        // the island needs few of them; first-fit colours only bound the colour count of islands
        // with long dependency chains (hundreds of levels), where one grid barrier per level and
        // iteration would dominate.
        int* col = color_.p;
        if (!exact && ncol <= tun_.exact_levels_colored) {
            int left_last = 0;
            PE_CK(cudaMemcpy(&left_last, gc_left_.p + ncol - 1, sizeof(int), cudaMemcpyDeviceToHost));
            if (left_last == 0) col = level;
        }
        PE_CK(cudaMemsetAsync(gc_cnt_.p, 0, (kMaxColorsBig + 1) * sizeof(int), st_));
        launch(K_GC_COLOR, g, k_gc_count, lo, m, col, gc_cnt_.p);
        PE_CK(cudaMemcpyAsync(cnt.data(), gc_cnt_.p, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaStreamSynchronize(st_));
        if (exact && cnt[kMaxColorsBig] > 0) {   // out of levels: the island in order on one thread
            launch_block(K_GC_SOLVE, 1, 1, k_isl_one<R>, lo, m, order, rs, jt, bd, rw, (const int*)row_off_.p, prm_.iterations);
            continue;
        }
        int run = 0, used = 0;
        for (int c = 0; c < kMaxColorsBig; c++) {
            start[c] = run; cur[c] = lo + run; run += cnt[c + 1];
            if (cnt[c + 1]) used = c + 1;
        }
        PE_CK(cudaMemcpyAsync(gc_cursor_.p, cur.data(), cur.size() * sizeof(int), cudaMemcpyHostToDevice, st_));
        launch(K_GC_COLOR, g, k_gc_place, lo, m, (const int*)col, order, gc_cursor_.p, isl_corder_.p);
        const bool last = cnt[kMaxColorsBig] > 0;
        n_colors_ = std::max(n_colors_, std::min(used, ncol) + (last ? 1 : 0));
        // every iteration in one cooperative launch: colour lists, then the grid-wide passes
        const int top = std::min(used, kMaxColorsBig - 1);
        std::vector<int> cs(std::max(top, 1)), cc(std::max(top, 1));
        for (int c = 0; c < top; c++) { cs[c] = lo + start[c]; cc[c] = cnt[c + 1]; }
        upload(gc_cstart_, cs, st_);
        upload(gc_ccount_, cc, st_);
        launch_coop(K_GC_SOLVE, coop_blocks_, kBlock, k_gc_solve<R>, (const uint32_t*)isl_corder_.p, (const int*)gc_cstart_.p,
                    (const int*)gc_ccount_.p, top, prm_.iterations, lo, m, order, (const int*)col, last ? 1 : 0, rs, jt, bd, rw,
                    (const int*)row_off_.p);
    }
}

// What a captured step graph holds fixed: buffer addresses (any reallocation changes the
// generation), sizes and capacities, the side-stream plan, the parameters and the settings.
// (Filled in place and compared bytewise: padding is zeroed here and copied with memcpy.)
template <class R> void World<R>::graph_sig(GraphSig& g) const {
    std::memset(&g, 0, sizeof g);
    g.gen = dbuf_generation().load();
    g.order = order_;
    g.n = N_; g.ns = NS_; g.pair_cap = pair_cap_; g.rows_cap = rows_cap_; g.nj = n_joints_; g.n_ign = n_ign_; g.s = S_;
    g.side = bcap_ * 4 + (max_scene_ > kBigWindow ? 1 : 0);
    std::memcpy(g.plan, stream_of_, sizeof g.plan);
    std::memcpy(&g.prm, &prm_, sizeof prm_);
    std::memcpy(&g.margin, &margin_, sizeof margin_);
    std::memcpy(&g.tun, &tun_, sizeof tun_);
}

// Replays `ex` if its signature `held` matches `sig`, else captures `enqueue` into it (updating the
// executable graph in place when the topology allows) once a step repeats its predecessor's
// signature `last`; until then `enqueue` launches directly.  Keeps the step's launch count.
template <class R>
template <class F>
void World<R>::graph_run(cudaGraphExec_t& ex, GraphSig& held, long long& held_launches, GraphSig& last, const GraphSig& sig, F&& enqueue) {
    const bool same_as_last = std::memcmp(&sig, &last, sizeof sig) == 0;
    std::memcpy(&last, &sig, sizeof sig);
    if (!ex || std::memcmp(&sig, &held, sizeof sig) != 0) {
        // a world that changes every step (a serving loop admitting and retiring scenes) would pay
        // a capture per step: capture only once the step has repeated its predecessor's settings
        if (!same_as_last) { enqueue(); return; }
        const long long before = step_launches_;
        cudaGraph_t g = nullptr;
        PE_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        capturing_ = true;
        try {
            enqueue();
        } catch (...) {
            capturing_ = false;
            cur_ = nullptr;
            cudaStreamEndCapture(st_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        capturing_ = false;
        PE_CK(cudaStreamEndCapture(st_, &g));
        cudaError_t e = cudaErrorUnknown;
        if (ex) {   // same topology (the usual case after a reallocation): update the executable graph in place
            cudaGraphExecUpdateResultInfo info;
            e = cudaGraphExecUpdate(ex, g, &info);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                cudaGraphExecDestroy(ex);
                ex = nullptr;
            }
        }
        if (!ex) e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { ex = nullptr; PE_CK(e); }
        std::memcpy(&held, &sig, sizeof sig);
        held_launches = step_launches_ - before;
        step_launches_ = before;
    }
    PE_CK(cudaGraphLaunch(ex, st_));
    step_launches_ += held_launches;
}

// The step's head (integration and the broadphase up to the pair count's copy to the host) as one
// CUDA graph; the host then waits for the count.
template <class R> void World<R>::run_head() {
    auto enqueue = [&]() {
        ev_begin(4);
        ev_begin(0); integrate(); ev_end(0);
        ev_begin(1);
        bp_count_enqueue();
    };
    if (!graphs_ || prof_) { enqueue(); return; }
    GraphSig sig;
    graph_sig(sig);
    graph_run(ghead_, gsig_head_, glaunch_head_, last_sig_head_, sig, enqueue);
}

// The step's device part after the pair count (pair list, narrowphase, solver): launched directly,
// or captured once as a CUDA graph per solver mode and contact-distance generation and replayed
// while nothing it holds fixed has changed.  The side-stream plan follows the last step's class
// counts; it is revised every 64 steps (a changed plan is a new capture).
template <class R> void World<R>::run_tail(int mode) {
    auto enqueue = [&]() {
        bp_tail();
        ev_end(1);
        ev_begin(2); np_enqueue(); ev_end(2);
        ev_begin(3); solve_enqueue(mode); ev_end(3);
        ev_end(4);
    };
    bool counted = false;
    for (int c = 0; c < PC_COUNT; c++) counted |= h_cls_[c] > 0;
    if (!graphs_ || prof_ || !counted) {   // no graph (or no class counts yet for the plan)
        plan_streams(stream_of_);
        enqueue();
        return;
    }
    const int m = mode ? 1 : 0, d = cur_dist_;
    if (!gexec_[m][d] || ++steps_since_plan_ >= 64) {
        steps_since_plan_ = 0;
        plan_streams(stream_of_);
    }
    GraphSig sig;
    graph_sig(sig);
    graph_run(gexec_[m][d], gsig_[m][d], glaunch_[m][d], last_sig_, sig, enqueue);
}

template <class R> void World<R>::step(int n, int mode) {
    for (int s = 0; s < n; s++) {
        step_launches_ = 0;
        run_head();
        PE_CK(cudaStreamSynchronize(st_));   // the first host wait: the pair count
        const int P = N_ < 2 ? P_ : hstat_[HS_P];
        prepare_tail(P);
        P_ = P;
        cur_dist_ ^= 1;
        run_tail(mode);
        R_ = P;
        finish(mode);               // the second
        ev_collect();
        last_step_launches_ = step_launches_;
    }
    resolve_prof();
}

} // namespace pe
