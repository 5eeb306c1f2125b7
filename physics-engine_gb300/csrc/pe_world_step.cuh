// World<R> member definitions, part 2: the step, phase by phase (sort and scan utilities,
// integrate, broadphase, narrowphase, solve, big islands).
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

template <class R> int World<R>::scan(int* data, int n) {
    const int tiles = (n + 1023) / 1024;
    if (tiles <= kSmallScanTiles) {   // small: one block scans in place (one launch instead of three)
        launch(K_SCAN, 1, k_scan_aux, data, n, total_.p);
    } else {
        aux_.ensure(tiles + 1);
        launch(K_SCAN, tiles, k_scan_tiles, data, n, aux_.p);
        launch(K_SCAN, 1, k_scan_aux, aux_.p, tiles, total_.p);
        launch(K_SCAN, tiles, k_scan_add, data, n, aux_.p);
    }
    int tot = 0;
    PE_CK(cudaMemcpyAsync(&tot, total_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    return tot;
}

template <class R> void World<R>::radix_sort(int n, int scene_passes) {
    order_ = val_[radix_sort_keys(n, (int)sizeof(R), scene_passes)].p;
}

template <class R> int World<R>::radix_sort_keys(int n, int key_passes, int scene_passes) {
    if (scene_passes == 0 && n <= kSceneSortMax) {   // small: one block, one launch
        launch_block(K_RADIX, 1, kSceneSortBlock, k_sort_pairs_block, (const uint64_t*)key_[0].p, (const uint32_t*)val_[0].p, n,
                     key_[1].p, val_[1].p);
        return 1;
    }
    const int tiles = (n + kRadixTile - 1) / kRadixTile;
    hist_.ensure((size_t)256 * tiles + 1);
    aux_.ensure((256 * tiles + 1023) / 1024 + 1);
    int cur = 0;
    auto pass = [&](int shift, int use2) {
        launch(K_RADIX, tiles, k_radix_hist, key_[cur].p, key2_[cur].p, n, shift, use2, hist_.p, tiles);
        const int m = 256 * tiles;
        const int st = (m + 1023) / 1024;
        if (st <= kSmallScanTiles) {
            launch(K_SCAN, 1, k_scan_aux, hist_.p, m, total_.p);
        } else {
            launch(K_SCAN, st, k_scan_tiles, hist_.p, m, aux_.p);
            launch(K_SCAN, 1, k_scan_aux, aux_.p, st, total_.p);
            launch(K_SCAN, st, k_scan_add, hist_.p, m, aux_.p);
        }
        launch(K_RADIX, tiles, k_radix_scatter, key_[cur].p, key2_[cur].p, val_[cur].p, key_[cur ^ 1].p, key2_[cur ^ 1].p,
                                                  val_[cur ^ 1].p, n, shift, use2, hist_.p, tiles);
        cur ^= 1;
    };
    for (int s = 0; s < key_passes * 8; s += 8) pass(s, 0);
    for (int s = 0; s < scene_passes * 8; s += 8) pass(s, 1);
    return cur;
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

template <class R> int World<R>::broadphase() {
    const int n = N_;
    if (n < 2) return P_;   // the reference leaves the pair list untouched below two bodies
    for (int k = 0; k < 2; k++) { key_[k].ensure(n); key2_[k].ensure(n); val_[k].ensure(n); }
    smn_.ensure((size_t)3 * n); smx_.ensure((size_t)3 * n); sflag_.ensure(n); ssc_.ensure(n);
    count_.ensure(n + 1);
    int max_scene = 0;
    for (int s = 0; s < NS_; s++) max_scene = std::max(max_scene, h_scene_off_[s + 1] - h_scene_off_[s]);
    if (max_scene <= std::min(tun_.scene_sort_max, kSceneSortMax)) {   // every scene sorted inside one block
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
    const bool crowded = max_scene > kBigWindow;
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
    const int P = scan(count_.p, n + 1);
    ensure_pair_capacity(P);
    launch(K_BP_SWEEP, grid_warps(n), k_bp_write<R>, n, scene_axis_.p, smn_.p, smx_.p, sflag_.p, ssc_.p, order_, count_.p, bp_stage_.p,
           pairs_.p, pair_cap_, status_.p, ign);
    if (crowded) launch(K_BP_SWEEP, 2 * kBigSweepBlocks, k_bp_write_chunks<R>, n, (const R*)smn_.p, (const R*)smx_.p, (const int*)sflag_.p,
           (const uint32_t*)order_, (const int*)count_.p, (const int*)bp_big_.p, (const int*)bp_nbig_.p, (const int*)bp_wend_.p,
           (const int*)bp_csize_.p, (const int*)bp_choff_.p, (const int*)bp_ctot_.p, (const int*)bp_cpref_.p, pairs_.p, pair_cap_,
           status_.p, ign);
    launch(K_MISC, grid(NS_ + 1), k_scene_pair_off, NS_, scene_off_.p, count_.p, n, pair_scene_off_.p);
    launch_block(K_BP_AXIS, NS_, 64, k_bp_axis<R>, (const R*)smn_.p, (const R*)smx_.p, n, (const int*)scene_off_.p, scene_axis_.p);
    PE_CK(cudaGetLastError());
    P_ = P;
    return P;
}

template <class R> void World<R>::narrowphase() {
    const int P = P_;
    ensure_pair_capacity(std::max(P, 1));
    // the results of the previous step become the pool the new step draws stale slots from
    PE_CK(cudaMemcpyAsync(prev_res_off_.p, res_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    cur_dist_ ^= 1;
    if (P > 0) {
        cls_count_.ensure(2 * PC_COUNT);
        PE_CK(cudaMemsetAsync(cls_count_.p, 0, 2 * PC_COUNT * sizeof(int), st_));
        launch(K_NP_BUCKET, grid(P), k_np_classify<R>, P, pairs_.p, bodies(), shapes(), cls_.p, cls_count_.p,
               (long long)tun_.sat_heavy_cost);
        int cnt[PC_COUNT];
        PE_CK(cudaMemcpyAsync(cnt, cls_count_.p, sizeof(cnt), cudaMemcpyDeviceToHost, st_));
        PE_CK(cudaStreamSynchronize(st_));
        int cur[PC_COUNT], run = 0;
        for (int c = 0; c < PC_COUNT; c++) { cur[c] = run; run += cnt[c]; }
        PE_CK(cudaMemcpyAsync(cls_count_.p + PC_COUNT, cur, sizeof(cur), cudaMemcpyHostToDevice, st_));
        launch(K_NP_BUCKET, grid(P), k_np_bucket, P, cls_.p, cls_count_.p + PC_COUNT, order_np_.p);
        const Results<R> rs = results();
        const Bodies<R> bd = bodies();
        const ShapeTable<R> sh = shapes();
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
        // The classes' kernels touch disjoint pairs and results: they run side by side on the side
        // streams, so the long tails of the serial per-pair kernels overlap the other classes.
        // Streams are given greedily, largest estimated work first (pairs x a rough per-pair cost).
        static_assert(PC_COUNT == 15, "one cost per pair class");
        static constexpr double kClassCost[PC_COUNT] = {2, 1, 1, 1, 4, 20, 6, 12, 400, 40, 40, 60, 20, 30, 30};
        int order_c[PC_COUNT], stream_of[PC_COUNT];
        double load[kSideStreams] = {};
        for (int c = 0; c < PC_COUNT; c++) order_c[c] = c;
        std::sort(order_c, order_c + PC_COUNT, [&](int a, int b) { return cnt[a] * kClassCost[a] > cnt[b] * kClassCost[b]; });
        for (int k = 0; k < PC_COUNT; k++) {
            const int c = order_c[k];
            const int best = (int)(std::min_element(load, load + kSideStreams) - load);
            stream_of[c] = best;
            load[best] += cnt[c] * kClassCost[c];
        }
        fork_streams();
        for (int c = 0; c < PC_COUNT; c++) {
            const int lo = cur[c], hi = cur[c] + cnt[c];
            if (hi == lo) continue;
            const int g = grid(hi - lo);
            use_stream(stream_of[c] % tun_.side_streams);
            switch (c) {
                case PC_BOX_BOX: launch(K_NP, g, k_np_class<R, PC_BOX_BOX>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_BOX_SPHERE: launch(K_NP, g, k_np_class<R, PC_BOX_SPHERE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_SPHERE: launch(K_NP, g, k_np_class<R, PC_SPHERE_SPHERE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_CYL: launch(K_NP, g, k_np_class<R, PC_SPHERE_CYL>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_BOX_CYL: launch(K_NP, g, k_np_class<R, PC_BOX_CYL>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p); break;
                case PC_SPHERE_HULL: {
                    const int w = sphere_hull_warps<R>();
                    launch_block(K_NP, (hi - lo + w - 1) / w, 32 * w, k_np_sphere_hull<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs,
                                 pair_scene_off_.p, prev_res_off_.p);
                    break;
                }
                case PC_CYL_HULL: {
                    const int w = cyl_hull_warps<R>();
                    launch_block(K_NP, (hi - lo + w - 1) / w, 32 * w, k_np_cyl_hull<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs,
                                 pair_scene_off_.p, prev_res_off_.p);
                    break;
                }
                case PC_CONVEX:
                case PC_CONVEX_HULL_BOX:
                case PC_CONVEX_HULL_HULL:
                case PC_CONVEX_CYL_CYL: {
                    const size_t smem = (size_t)kSatWarps * sat_group_reals<R>(1) * sizeof(R);
                    const int gb = (hi - lo + kSatWarps - 1) / kSatWarps, bs = 32 * kSatWarps;
                    auto kern = c == PC_CONVEX ? k_np_sat<R, 1, ST_BOX, ST_HULL>
                              : c == PC_CONVEX_HULL_BOX ? k_np_sat<R, 1, ST_HULL, ST_BOX>
                              : c == PC_CONVEX_HULL_HULL ? k_np_sat<R, 1, ST_HULL, ST_HULL>
                              : k_np_sat<R, 1, ST_CYLINDER, ST_CYLINDER>;
                    launch_smem(K_NP_SAT, gb, bs, smem, kern, lo, hi, order_np_.p, pairs_.p, bd, sh, sat_out_.p);
                    launch(K_NP_SAT, grid(hi - lo), k_np_sat_finish<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p, (const R*)sat_out_.p);
                    break;
                }
                case PC_CONVEX_HEAVY: {
                    const size_t smem = (size_t)sat_group_reals<R>(kSatGroup) * sizeof(R);
                    launch_smem(K_NP_SAT, hi - lo, 32 * kSatGroup, smem, k_np_sat<R, kSatGroup, -1, -1>, lo, hi, order_np_.p, pairs_.p, bd,
                                sh, sat_out_.p);
                    launch(K_NP_SAT, grid(hi - lo), k_np_sat_finish<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p, (const R*)sat_out_.p);
                    break;
                }
                case PC_COMPOUND:
                    launch(K_NP, g, k_np_compound<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p, prev_res_off_.p);
                    break;
                case PC_CONCAVE:
                    launch(K_NP, g, k_np_class<R, PC_CONCAVE>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs, pair_scene_off_.p,
                           prev_res_off_.p);
                    break;
                default:   // PC_CONVEX_BIG
                    launch(K_NP_SAT, grid_warps(hi - lo), k_np_sat_big<R>, lo, hi, order_np_.p, pairs_.p, bd, sh, rs,
                           pair_scene_off_.p, prev_res_off_.p);
                    break;
            }
        }
        join_streams();
        PE_CK(cudaGetLastError());
    }
    PE_CK(cudaMemcpyAsync(res_scene_off_.p, pair_scene_off_.p, (NS_ + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
    R_ = P;
}

template <class R> void World<R>::solve(int mode) {
    const int P = R_;
    if (N_ == 0) return;
    launch(K_SI_MISC, grid(N_), k_si_clear<R>, bodies());
    n_active_ = 0;
    n_colors_ = 0;
    n_islands_ = 0;
    if (P > 0) {
        // rows: one per contact point, results' rows contiguous in result order
        PE_CK(cudaMemcpyAsync(row_off_.p, res_np_.p, P * sizeof(int), cudaMemcpyDeviceToDevice, st_));
        PE_CK(cudaMemsetAsync(row_off_.p + P, 0, sizeof(int), st_));
        // a result has at most kSlots points, so kSlots * P rows always fit: the row total is read
        // back with the step's status at its end instead of in a host wait here
        if ((long long)kSlots * P > rows_cap_) {
            rows_cap_ = std::max(kSlots * P + kSlots * P / 4, 1024);
            rows_.ensure((size_t)NRF * rows_cap_);
        }
        scan_async(row_off_.p, P + 1, rows_total_.p);
        PE_CK(cudaMemcpyAsync(h_rows_, rows_total_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
        rows_pending_ = true;
        launch(K_SI_SETUP, grid(P), k_si_setup<R>, P, results(), bodies(), rows(), row_off_.p, prm_, status_.p);
        // results with points, in result order
        launch(K_SI_MISC, grid(P + 1), k_active_flags, P, res_np_.p, active_.p);
        color_.ensure(P + 1);
        PE_CK(cudaMemcpyAsync(color_.p, active_.p, (P + 1) * sizeof(int), cudaMemcpyDeviceToDevice, st_));
        n_active_ = scan(color_.p, P + 1);
        launch(K_SI_MISC, grid(P), k_active_compact, P, res_np_.p, color_.p, active_.p);
    }
    const int A = n_active_, NJ = n_joints_;
    const Joints<R> jt = joints();
    if (NJ > 0) launch(K_SI_SETUP, grid(NJ), k_joint_init<R>, jt, bodies(), prm_);
    const int M = A + NJ;   // island items: active contact results, then joints
    if (M > 0) {
        // islands: union-find over dynamic bodies linked by contacts and joints; items grouped by
        // island keeping their order (contacts in result order, then joints in order)
        parent_.ensure(N_ + 1);
        launch(K_ISLAND, grid(N_), k_isl_init, N_, parent_.p);
        if (A > 0) launch(K_ISLAND, grid(A), k_isl_union<R>, A, active_.p, results(), bodies(), parent_.p);
        if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_union_joints<R>, jt, bodies(), parent_.p);
        for (int k = 0; k < 2; k++) { key_[k].ensure(M); key2_[k].ensure(M); val_[k].ensure(M); }
        if (A > 0)
            launch(K_ISLAND, grid(A), k_isl_keys<R>, A, active_.p, results(), bodies(), parent_.p, key_[0].p, key2_[0].p, val_[0].p);
        if (NJ > 0) launch(K_ISLAND, grid(NJ), k_isl_keys_joints<R>, jt, bodies(), parent_.p, A, key_[0].p, key2_[0].p, val_[0].p);
        int label_passes = 0;
        for (int m = NJ > 0 ? N_ : N_ - 1; m > 0; m >>= 8) label_passes++;   // joint labels reach n_bodies
        const int cur = radix_sort_keys(M, label_passes, 0);
        const uint64_t* skey = key_[cur].p;
        const uint32_t* order = val_[cur].p;
        isl_flag_.ensure(M + 1);
        isl_off_.ensure(M + 1);
        isl_n_.ensure(1);
        launch(K_ISLAND, grid(M + 1), k_isl_flags, M, skey, isl_flag_.p);
        n_islands_ = scan(isl_flag_.p, M + 1);
        launch(K_ISLAND, grid(M + 1), k_isl_offsets, M, skey, isl_flag_.p, isl_off_.p, isl_n_.p);
        const int NI = n_islands_;
        // islands of up to small_island_items items: one thread each
        launch(K_SI_SERIAL, grid(NI), k_isl_serial<R>, (const int*)isl_n_.p, (const int*)isl_off_.p, order, results(), jt, bodies(),
               rows(), (const int*)row_off_.p, prm_.iterations, tun_.small_island_items);
        if (mode == 0) {
            // serial order, larger islands: the exact level schedule, a block per island up to
            // big_island_items items, grid-wide above
            isl_corder_.ensure(M);
            color_.ensure(M + 1);
            launch_block(K_SI_SERIAL, NI, tun_.level_block, k_isl_levels<R>, isl_n_.p, isl_off_.p, order, results(), jt, bodies(), rows(),
                         row_off_.p, prm_.iterations, tun_.small_island_items, tun_.big_island_items, claim_.p, color_.p, isl_corder_.p);
            solve_big_islands(NI, order, true);
        } else {
            isl_corder_.ensure(M);
            color_.ensure(M + 1);
            ncol_.ensure(1);
            PE_CK(cudaMemsetAsync(ncol_.p, 0, sizeof(int), st_));
            launch_block(K_SI_COLOR, NI, tun_.color_block, k_isl_colored<R>, isl_n_.p, isl_off_.p, order, results(), jt, bodies(), rows(),
                         row_off_.p, prm_.iterations, tun_.small_island_items, tun_.big_island_items, claim_.p, color_.p, isl_corder_.p,
                         ncol_.p);
            PE_CK(cudaMemcpyAsync(&n_colors_, ncol_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
            solve_big_islands(NI, order, false);
        }
    }
    launch(K_SI_MISC, grid(N_), k_si_sync<R>, bodies());
    PE_CK(cudaGetLastError());
}

// islands above big_island_items results: grid-wide colouring rounds, then one launch per
// colour and iteration (see k_gc_*)
template <class R> void World<R>::solve_big_islands(int NI, const uint32_t* order, bool exact) {
    gc_big_.ensure(NI + 1);
    gc_n_.ensure(2);
    PE_CK(cudaMemsetAsync(gc_n_.p, 0, sizeof(int), st_));
    launch(K_SI_COLOR, grid(NI), k_isl_big, (const int*)isl_n_.p, (const int*)isl_off_.p, gc_big_.p, gc_n_.p, tun_.big_island_items);
    int nb = 0;
    PE_CK(cudaMemcpyAsync(&nb, gc_n_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    PE_CK(cudaStreamSynchronize(st_));
    if (nb == 0) return;
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

template <class R> void World<R>::step(int n, int mode) {
    for (int s = 0; s < n; s++) {
        step_launches_ = 0;
        ev_begin(4);
        ev_begin(0); integrate(); ev_end(0);
        ev_begin(1); broadphase(); ev_end(1);
        ev_begin(2); narrowphase(); ev_end(2);
        ev_begin(3); solve(mode); ev_end(3);
        ev_end(4);
        last_step_launches_ = step_launches_;
        check_status();
    }
    resolve_prof();
}

} // namespace pe
