// tc_kernel.cuh -- the tcgen05 mainloop + epilogues of the genotype operator.
//
// One CTA owns a 128-row tile (K1: 128 SNP slots, K2: 128 samples) and walks
// K in stages of Cfg::SB x 64 (K1: samples, K2: SNP slots).  Per stage:
//   warp 0   bulk-copies the Cfg::SB consecutive 2 KB genotype blocks into
//            a shared ring;
//   warp 2   bulk-copies the B tile (all split terms of V or S for these 64
//            K values) into a shared ring;
//   warp 3   idles (the CTA is a whole number of warpgroups);
//   warps 4.. decode in Cfg::SETS sets of 4 warps (one per tensor-memory lane
//            quarter); a set turns the 16-byte rows (64 codes) of one chunk
//            into 32 BF16 pairs per row stored with tcgen05.st into an A ring
//            in tensor memory, and the sets take successive chunks so that
//            several store round trips are in flight;
//   warp 1   lane 0 issues the MMAs.  With SIDE the split terms sit side by
//            side in N (one MMA of N = NSPLIT*kp per 16-wide K step, the
//            epilogue sums the column groups); otherwise each term is its own
//            MMA into one accumulator.
// Barrier arrivals from the decoders are per warp.  All waits are bounded.
//
// Split K: with p.ksplit > 1 the CTA at blockIdx.z walks only its share of
// the stages and writes its FP32 partial (split terms summed) to p.part; a
// finish kernel sums the partials and applies the epilogue.  Tensor-core FP32
// accumulation loses precision over very long chains (relative error grows
// with the number of MMAs into one accumulator), so the host bounds every
// chain this way.
//
// Two tiles per CTA (TILES = 2): the CTA owns two consecutive row tiles of
// the same K share, which read the same B tile at every stage.  One genotype
// ring slot holds both tiles' blocks of a stage, each decoder warp decodes
// its rows of both tiles into one A-ring slot (tile 0's blocks, then tile
// 1's), and two threads issue the MMAs -- lane 0 of warp 1 for tile 0 into
// accumulator 0, lane 0 of warp 3 for tile 1 into accumulator 1 -- so the
// SM runs two instruction streams (one thread pays a fixed ~120 cycles per
// tcgen05.mma whatever N is) on one B supply.  A and B slots are released
// when both issuers' commits have arrived.  A padding tile (odd tile count)
// repeats the last tile without writing results.
//
// Clusters (CL > 1): the CL CTAs of a cluster own consecutive tiles of the
// same K share and so read the same B tile at every stage.  Each copies 1/CL
// of the stage into the B ring of every CTA of the cluster (bulk copy with
// cluster multicast, within this GPU's memory), which divides the B traffic
// from L2 by CL; a B slot is refilled once every CTA's MMAs are done with it
// (each MMA thread's commit arrives on that slot's empty barrier in every
// CTA, so the barrier counts CL arrivals).  A CTA leaves only after the last
// arrivals of the other CTAs on its own barriers have landed.  The grid is a
// whole number of clusters; a padding CTA repeats the last tile without
// writing results.

template <bool IS_K1, int NSPLIT, bool SIDE, class Cfg, int TY, int CL, int TILES>
__global__ void __launch_bounds__(Cfg::THREADS, 1) k_tc_op(const __grid_constant__ TcParams p) {
  static_assert(TILES == 1 || TILES == 2, "one or two tiles per CTA");
  constexpr int kStageBlocks = Cfg::SB;
  // Tensor-memory columns of one 64-K block of A: 32 for 16-bit operands,
  // 16 for E4M3 bytes.
  constexpr uint32_t kACols = TY == kTyE4M3 ? 16u : 32u;
  constexpr int kSets = Cfg::SETS;
  constexpr int kMaxRG = Cfg::RG;  // barrier slots; the ring itself holds p.RG stages
  extern __shared__ __align__(1024) uint8_t smem[];
  uint64_t* fullG = reinterpret_cast<uint64_t*>(smem);
  uint64_t* emptyG = fullG + kMaxRG;
  uint64_t* fullB = emptyG + kMaxRG;
  uint64_t* emptyB = fullB + kMaxRB;
  uint64_t* decoded = emptyB + kMaxRB;
  uint64_t* emptyA = decoded + kMaxRA;
  uint64_t* done = emptyA + kMaxRA;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  constexpr int kStageBytes = kStageBlocks * kBlockBytes;   // one tile's blocks of a stage
  constexpr int kGSlotBytes = TILES * kStageBytes;           // a genotype ring slot
  uint8_t* gring = smem + kBarrierBytes;
  const int kRG = p.RG;
  uint8_t* bring = gring + kRG * kGSlotBytes;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const EpiParams& e = p.e;
  const int kp = e.kp;
  const int RA = p.RA;
  const int RB = p.RB;

  // Tile t of this CTA: row tile blockIdx.x * TILES + t (padding tiles past
  // the last one repeat it and write nothing).
  int64_t tile[TILES];
  bool active[TILES];
#pragma unroll
  for (int t = 0; t < TILES; ++t) {
    const int64_t tt = static_cast<int64_t>(blockIdx.x) * TILES + t;
    active[t] = tt < p.n_tiles;
    tile[t] = active[t] ? tt : p.n_tiles - 1;
  }
  const int comp = blockIdx.y;
  constexpr uint16_t kClusterMask = static_cast<uint16_t>((1u << CL) - 1u);
  const int zsplit = blockIdx.z;
  int64_t ntot;
  const uint8_t* gbase[TILES];
  const uint8_t* bbase;
  const int64_t stage_b_bytes = kStageBlocks * p.b_chunk_bytes;
  // Stages of kStageBlocks consecutive 2 KB blocks along K.
  if (IS_K1) {
    ntot = p.n_chunks / kStageBlocks;
#pragma unroll
    for (int t = 0; t < TILES; ++t) gbase[t] = p.geno + tile[t] * p.n_chunks * kBlockBytes;
    bbase = p.bsrc;
  } else {
    int64_t p0 = 0, p1 = p.n_panels;
    if (e.stacked) {
      p0 = p.comp_slot_start[comp] / kPanel;
      p1 = p.comp_slot_start[comp + 1] / kPanel;
    }
    ntot = (p1 - p0) / kStageBlocks;
#pragma unroll
    for (int t = 0; t < TILES; ++t) gbase[t] = p.geno + (tile[t] * p.n_panels + p0) * kBlockBytes;
    bbase = p.bsrc + p0 * p.b_chunk_bytes;
  }
  // This CTA's share of the K stages: [s0, s0 + nch).  The host keeps a
  // share at most 65,536 K values long (split K), so 32-bit stage counters
  // hold.
  const int64_t s0 = ntot * zsplit / p.ksplit;
  const int nch = static_cast<int>(ntot * (zsplit + 1) / p.ksplit - s0);
#pragma unroll
  for (int t = 0; t < TILES; ++t) gbase[t] += s0 * kStageBytes;
  bbase += s0 * stage_b_bytes;

  if (threadIdx.x == 0) {
    // Each chunk is consumed and decoded by one set of 4 warps.
    for (int i = 0; i < kMaxRG; ++i) {
      ptx::mbar_init(&fullG[i], 1);
      ptx::mbar_init(&emptyG[i], 4);
    }
    // Empty barriers of the A and B rings and `done` count one commit per
    // issuing thread (per CTA of the cluster for B).
    for (int i = 0; i < kMaxRB; ++i) {
      ptx::mbar_init(&fullB[i], 1);
      ptx::mbar_init(&emptyB[i], CL * TILES);
    }
    for (int i = 0; i < kMaxRA; ++i) {
      ptx::mbar_init(&decoded[i], 4);
      ptx::mbar_init(&emptyA[i], TILES);
    }
    ptx::mbar_init(done, TILES);
    *abort_flag = 0;
    ptx::fence_barrier_init();
  }
  // Self-check of the launch configuration: every tensor-memory column the
  // CTA touches (accumulator + A ring) must lie inside its allocation, and the
  // rings must fit their barrier arrays; otherwise record an error and exit
  // before touching tensor memory.
  {
    const uint32_t acc_need = SIDE ? static_cast<uint32_t>(NSPLIT * e.kp) : static_cast<uint32_t>(e.kp);
    // RA >= kSets: a decoder set never waits on an A slot whose previous use
    // is more than one barrier phase behind (parity waits are ambiguous
    // beyond one phase).
    const bool cfg_ok = p.RA >= kSets && p.RA >= Cfg::MIN_RA && p.RA <= kMaxRA && p.RB >= 1 &&
                        kRG >= kSets && kRG <= kMaxRG && kRG % kSets == 0 &&
                        p.RB <= kMaxRB &&
                        p.ksplit >= 1 && static_cast<int>(gridDim.z) == p.ksplit &&
                        (p.ksplit == 1 || p.part != nullptr) &&
                        acc_need <= p.acc_cols && (p.acc_cols & 31u) == 0 &&
                        TILES * p.acc_cols +
                                static_cast<uint32_t>(p.RA) * kACols * kStageBlocks * TILES <=
                            p.tmem_cols &&
                        p.tmem_cols >= 32 && p.tmem_cols <= 512 &&
                        (p.tmem_cols & (p.tmem_cols - 1)) == 0 && acc_need <= 256 && (e.kp & 15) == 0 &&
                        p.n_tiles >= 1 && p.n_tiles <= static_cast<int64_t>(gridDim.x) * TILES &&
                        gridDim.x % CL == 0 && p.bslot_bytes % (16u * CL) == 0;
    if (!cfg_ok) {
      if (threadIdx.x == 0) atomicCAS(p.err, 0, 30);
      return;
    }
  }
  if (warp == kWarpMMA) ptx::tmem_alloc(tmem_slot, p.tmem_cols);
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  // Every CTA of the cluster has initialised its barriers before any copy or
  // commit reaches them.
  if constexpr (CL > 1) ptx::cluster_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == kWarpG) {
    // ---------------------------------------------- genotype block producer
    if (lane == 0) {
      // Ring slot and phase parity are carried as counters: no division in
      // the per-stage loops of the single-thread roles.
      int issued = 0;
      int s = 0;
      uint32_t ph = 0;
      for (int c = 0; c < nch; ++c) {
        if (c >= kRG && !ptx::mbar_wait(&emptyG[s], ph ^ 1u, p.err, 11, abort_flag)) break;
        ptx::mbar_arrive_expect_tx(&fullG[s], kGSlotBytes);
#pragma unroll
        for (int t = 0; t < TILES; ++t)
          ptx::bulk_g2s(gring + s * kGSlotBytes + t * kStageBytes,
                        gbase[t] + static_cast<int64_t>(c) * kStageBytes, kStageBytes, &fullG[s]);
        issued = c + 1;
        if (++s == kRG) { s = 0; ph ^= 1u; }
      }
      if (*abort_flag) {
        // Let copies still in flight land before the CTA exits.
        for (int c = (issued > kRG ? issued - kRG : 0); c < issued; ++c) {
          volatile int no_abort = 0;
          ptx::mbar_wait(&fullG[c % kRG], static_cast<uint32_t>(c / kRG) & 1, p.err, 18,
                         &no_abort);
        }
      }
    }
  } else if (warp == kWarpB) {
    // ---------------------------------------------------- B tile producer
    if (lane == 0) {
      int issued = 0;
      int s = 0;
      uint32_t ph = 0;
      const uint32_t share = p.bslot_bytes / CL;
      const uint32_t own = CL > 1 ? ptx::cluster_ctarank() * share : 0u;
      for (int c = 0; c < nch; ++c) {
        if (c >= RB && !ptx::mbar_wait(&emptyB[s], ph ^ 1u, p.err, 12, abort_flag)) break;
        // The full slot arrives on this CTA's barrier: its own share and the
        // shares the other CTAs of the cluster multicast.
        ptx::mbar_arrive_expect_tx(&fullB[s], p.bslot_bytes);
        if constexpr (CL > 1)
          ptx::bulk_g2s_multicast(bring + static_cast<size_t>(s) * p.bslot_bytes + own,
                                  bbase + static_cast<int64_t>(c) * stage_b_bytes + own, share,
                                  &fullB[s], kClusterMask);
        else
          ptx::bulk_g2s(bring + static_cast<size_t>(s) * p.bslot_bytes,
                        bbase + static_cast<int64_t>(c) * stage_b_bytes, p.bslot_bytes, &fullB[s]);
        issued = c + 1;
        if (++s == RB) { s = 0; ph ^= 1u; }
      }
      if constexpr (CL > 1) {
        // The other CTAs' commits for the last use of every slot arrive on
        // this CTA's barriers: wait for them before the CTA may exit.
        if (!*abort_flag)
          for (int c = (nch > RB ? nch - RB : 0); c < nch; ++c)
            if (!ptx::mbar_wait(&emptyB[c % RB], static_cast<uint32_t>(c / RB) & 1u, p.err, 21,
                                abort_flag))
              break;
      }
      if (*abort_flag) {
        for (int c = (issued > RB ? issued - RB : 0); c < issued; ++c) {
          volatile int no_abort = 0;
          ptx::mbar_wait(&fullB[c % RB], static_cast<uint32_t>(c / RB) & 1, p.err, 19, &no_abort);
        }
      }
    }
  } else if (warp == kWarpMMA || (TILES == 2 && warp == kWarpIdle)) {
    // ------------------------------------------------------------ MMA issue
    // Warp 1 issues tile 0's MMAs, warp 3 (two tiles per CTA) tile 1's.
    const int mt = warp == kWarpMMA ? 0 : 1;
    if (lane == 0) {
      const int nn = SIDE ? NSPLIT * kp : kp;
      const uint32_t idesc = TY == kTyE4M3 ? ptx::idesc_e4m3_f32(128, nn)
                             : TY == kTyF16 ? ptx::idesc_f16_f32(128, nn)
                                            : ptx::idesc_bf16_f32(128, nn);
      // B tiles: core matrices of 8 columns x 16 bytes; a 64-K block holds
      // 8 (16-bit) or 4 (8-bit) of them per 8-column group.
      const uint64_t bdesc0 =
          ptx::smem_desc(ptx::smem_addr(bring), 128u, TY == kTyE4M3 ? 512u : 1024u);
      const uint32_t term_off = static_cast<uint32_t>(kp * 128) >> 4;
      int as = 0, bs = 0;
      uint32_t pa = 0, pb = 0;
      for (int c = 0; c < nch; ++c) {
        if (!ptx::mbar_wait(&decoded[as], pa, p.err, 13, abort_flag)) break;
        if (!ptx::mbar_wait(&fullB[bs], pb, p.err, 14, abort_flag)) break;
        ptx::tc_fence_after();
        const uint64_t bslot = bdesc0 + ((static_cast<uint64_t>(bs) * p.bslot_bytes) >> 4);
        const uint32_t a_slot = tmem + TILES * p.acc_cols +
                                static_cast<uint32_t>(as * TILES + mt) * (kACols * kStageBlocks);
        const uint32_t dacc = tmem + static_cast<uint32_t>(mt) * p.acc_cols;
        const uint32_t first = c == 0 ? 0u : 1u;
#pragma unroll
        for (int b = 0; b < kStageBlocks; ++b) {
          const uint64_t bblk = bslot + ((static_cast<uint64_t>(b) * p.b_chunk_bytes) >> 4);
          const uint32_t a_col = a_slot + kACols * b;
          // K steps of one 64-K block: 4 of 16 (16-bit) or 2 of 32 (E4M3);
          // each advances A by 8 columns and B by two 16-byte core matrices.
#pragma unroll
          for (int ks = 0; ks < (TY == kTyE4M3 ? 2 : 4); ++ks) {
            const uint32_t acc0 = (b == 0 && ks == 0) ? first : 1u;
            if (TY == kTyE4M3) {
              ptx::mma_ts_f8(dacc, a_col + ks * 8, bblk + ks * 16, idesc, acc0);
            } else if (SIDE) {
              ptx::mma_ts(dacc, a_col + ks * 8, bblk + ks * 16, idesc, acc0);
            } else {
#pragma unroll
              for (int t = 0; t < NSPLIT; ++t)
                ptx::mma_ts(dacc, a_col + ks * 8, bblk + ks * 16 + t * term_off, idesc,
                            t == 0 ? acc0 : 1u);
            }
          }
        }
        ptx::mma_commit(&emptyA[as]);
        if constexpr (CL > 1)
          ptx::mma_commit_multicast(&emptyB[bs], kClusterMask);
        else
          ptx::mma_commit(&emptyB[bs]);
        if (++as == RA) { as = 0; pa ^= 1u; }
        if (++bs == RB) { bs = 0; pb ^= 1u; }
      }
      if (nch == 0) {
        ptx::mbar_arrive(done);
      } else {
        ptx::mma_commit(done);
      }
      if (*abort_flag) {
        // Tensor memory is released below: let issued MMAs finish first.
        volatile int no_abort = 0;
        ptx::mbar_wait(done, 0, p.err, 20, &no_abort);
      }
    }
  } else if (warp == kWarpIdle) {
    // One tile per CTA: pads the CTA to whole warpgroups (see StageCfg::THREADS).
  } else {
    // --------------------------------------------- decoders, then epilogue
    // Decoder warp sets: set s handles chunks s, s + kSets, ...; within a set
    // the 4 warps cover the 4 tensor-memory lane quarters (128 rows).
    const int dw = warp - kWarpDec0;
    const int quarter = warp & 3;
    const int set = dw >> 2;
    const int row = quarter * 32 + lane;
    const uint32_t lane_base = static_cast<uint32_t>(quarter * 32) << 16;
    bool ok = true;
    // Stage c = set + i * kSets: its G slot/phase and A slot/round advance by
    // kSets per step (kSets <= kRG and kSets <= RA, so one wrap at most).
    int gs = set, as = set;
    uint32_t gph = 0, around = 0;
    for (int c = set; c < nch; c += kSets) {
      bool w_ok = ptx::mbar_wait(&fullG[gs], gph, p.err, 15, abort_flag);
      if (!__all_sync(0xffffffffu, w_ok)) { ok = false; break; }
      uint4 raw[TILES][kStageBlocks];
#pragma unroll
      for (int t = 0; t < TILES; ++t)
#pragma unroll
        for (int b = 0; b < kStageBlocks; ++b)
          raw[t][b] = *reinterpret_cast<const uint4*>(gring + gs * kGSlotBytes + t * kStageBytes +
                                                      b * kBlockBytes + row * kRowBytes);
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&emptyG[gs]);
      if (c >= RA) {
        w_ok = ptx::mbar_wait(&emptyA[as], (around - 1u) & 1u, p.err, 16, abort_flag);
        if (!__all_sync(0xffffffffu, w_ok)) { ok = false; break; }
      }
      ptx::tc_fence_after();
#pragma unroll
      for (int t = 0; t < TILES; ++t)
#pragma unroll
        for (int b = 0; b < kStageBlocks; ++b) {
          const uint32_t col =
              tmem + lane_base + TILES * p.acc_cols +
              static_cast<uint32_t>((as * TILES + t) * kStageBlocks + b) * kACols;
          if constexpr (TY == kTyE4M3) {
            uint32_t a[16];
            decode_row_e4m3(raw[t][b], a);
            ptx::tmem_st16(col, a);
          } else {
            uint32_t a[32];
            decode_row<TY == kTyF16>(raw[t][b], a);
            ptx::tmem_st32(col, a);
          }
        }
      ptx::tmem_wait_st();
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) ptx::mbar_arrive(&decoded[as]);
      gs += kSets;
      if (gs >= kRG) { gs -= kRG; gph ^= 1u; }
      as += kSets;
      if (as >= RA) { as -= RA; ++around; }
    }
    if (ok) {
      const bool w_ok = ptx::mbar_wait(done, 0, p.err, 17, abort_flag);
      ok = __all_sync(0xffffffffu, w_ok);
    }
    if (ok) {
      ptx::tc_fence_after();
#pragma unroll
      for (int t = 0; t < TILES; ++t) {
        if (!active[t]) continue;
        const int64_t rowid = tile[t] * kTile + row;
        const uint32_t acc = tmem + lane_base + static_cast<uint32_t>(t) * p.acc_cols;
        // Column chunks of 16 rotate over the kSets warps of a quarter.
        for (int c0 = 16 * set; c0 < kp; c0 += 16 * kSets) {
          float T[16];
          if (nch > 0) {
            uint32_t r[16];
            ptx::tmem_ld16(acc + static_cast<uint32_t>(c0), r);
            ptx::tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 16; ++i) T[i] = __uint_as_float(r[i]);
            if (SIDE) {
              // Terms side by side: 16-bit terms share one scale; E4M3 term
              // u carries 16^u (each holds the previous residual times 16).
#pragma unroll
              for (int u = 1; u < NSPLIT; ++u) {
                ptx::tmem_ld16(acc + static_cast<uint32_t>(u * kp + c0), r);
                ptx::tmem_wait_ld();
                const float wt = TY == kTyE4M3 ? ldexpf(1.f, -4 * u) : 1.f;
#pragma unroll
                for (int i = 0; i < 16; ++i) T[i] = fmaf(wt, __uint_as_float(r[i]), T[i]);
              }
            }
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) T[i] = 0.f;
          }
          if (p.ksplit > 1) {
            // Partial of this K share: row (K1: slot; K2: component, sample).
            const int64_t prow =
                IS_K1 ? rowid : static_cast<int64_t>(comp) * p.part_rows + rowid;
            float4* dst =
                reinterpret_cast<float4*>(p.part + zsplit * p.part_stride + prow * kp + c0);
#pragma unroll
            for (int q = 0; q < 4; ++q)
              dst[q] = make_float4(T[4 * q], T[4 * q + 1], T[4 * q + 2], T[4 * q + 3]);
          } else if (IS_K1) {
            epilogue_k1(e, rowid, c0, T, lane);
          } else {
            epilogue_k2(e, rowid, comp, c0, T);
          }
        }
      }
    }
  }

  ptx::tc_fence_before();
  __syncthreads();
  if (warp == kWarpMMA) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, p.tmem_cols);
  }
}
