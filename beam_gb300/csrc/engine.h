// Host runtime of the GB300 merge loop: owns the device-resident graph,
// quotient graph, partition lists and per-block scratch, and sequences the
// kernels of Sweg::Run (src/sweg.cpp:651-709) on one CUDA stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.cuh"

namespace beam {

struct EncodeOutput;

struct EngineConfig {
  int top_k = 16;
  int group_batch_size = 64;
  int divide_hash_dims = 16;
  int divide_max_group = 512;
  bool ea_use_threshold = true;
  uint64_t seed = 1;
  int device = 0;
  // Re-score every selected pair at commit and check it (--verify-cuda-gain).
  bool verify_cuda_gain = false;
  // Learned candidate ranker (off: the reference's method).
  bool ranker = false;
  int ranker_train_iters = 5;
  float ranker_recall = 0.99f;
  bool ranker_audit = false;
  int ranker_max_samples = 1 << 18;
  int ranker_epochs = 4;
  int ranker_max_steps = 256;
  float ranker_lr = 3e-3f;
};

struct RankerInfo {
  uint64_t samples = 0, positives = 0, train_steps = 0;
  double train_ms = 0, first_loss = 0, final_loss = 0, cutoff = 0, calib_recall = 0, calib_prune = 0;
  bool trained = false;
};

// Largest group the kernels accept (bounded by the packed select keys and
// the per-group pair tables); the reference default is 512.
constexpr int kMaxGroup = 1024;
// Persistent grid of the row-update kernels (four CTAs per SM of a GB300).
constexpr int kRowsGrid = 4 * 152;

void CheckCuda(cudaError_t status, const char* what);

// Device memory. Inside an AllocScope (every engine call sets one for its
// stream) buffers come from the device's stream-ordered pool, which keeps
// freed memory for the next allocation, so creating, growing and destroying
// engines pays no cudaMalloc / cudaFree; outside one, plain cudaMalloc.
cudaStream_t CurrentAllocStream();
void* DeviceAlloc(size_t bytes, cudaStream_t s);
void DeviceFree(void* p, cudaStream_t s);

class AllocScope {
 public:
  explicit AllocScope(cudaStream_t s);
  ~AllocScope();
  AllocScope(const AllocScope&) = delete;
  AllocScope& operator=(const AllocScope&) = delete;

 private:
  cudaStream_t prev_;
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // stream of a pool allocation (nullptr: cudaMalloc)
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void ensure(size_t count) {
    if (count <= n) return;
    release();
    const size_t bytes = (count ? count : 1) * sizeof(T);
    s = CurrentAllocStream();
    p = static_cast<T*>(DeviceAlloc(bytes, s));
    n = count;
  }
  void release() {
    if (p) DeviceFree(p, s);
    p = nullptr;
    n = 0;
    s = nullptr;
  }
};

// The engine's stream, destroyed after every buffer of the engine is freed
// (declared before them).
struct OwnedStream {
  cudaStream_t s = nullptr;
  OwnedStream() = default;
  OwnedStream(const OwnedStream&) = delete;
  OwnedStream& operator=(const OwnedStream&) = delete;
  ~OwnedStream() {
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
};

template <typename T>
struct PinnedBuf {
  T* p = nullptr;
  size_t n = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { release(); }
  void ensure(size_t count) {
    if (count <= n) return;
    release();
    CheckCuda(cudaMallocHost(reinterpret_cast<void**>(&p), (count ? count : 1) * sizeof(T)), "cudaMallocHost");
    n = count;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

// Per-block control words, reset before every 64-group block.
struct BlockCtl {
  unsigned long long scratch_top;  // bump pointer into the block scratch (bytes)
  unsigned int short_cnt;   // claimed neighbour rows rewritten by one warp each
  unsigned int long_cnt;    // claimed neighbour rows rewritten by one CTA each
  unsigned int sel_total;   // selected pairs of the block (entries of the selection list)
  unsigned int pad;
  // work queues of the dynamically scheduled kernels: the accumulate pass and
  // the two scoring passes (exploration / the rest, or the only one)
  unsigned long long work_next[3];
};

// One block of an iteration's plan: its real-group range, its candidate and
// selection slots, and the ranges of the prepare and select lists covering it.
struct BlockPlan {
  int rg0 = 0, rg1 = 0;                 // real-group positions
  long long slots = 0, sel_slots = 0;   // candidate / selection slots
  int s0 = 0, s1 = 0, b0 = 0, b1 = 0;   // small / big prepare list ranges
  long long members = 0;                // members of the big groups
  long long slot0 = 0, nslots = 0;      // sort slots of the deferred big groups
  long long max_e = 0;                  // largest deferred group's row entries
  long long mat_bytes = 0;              // pair tables of the big groups
  int ss0 = 0, ss1 = 0, sm0 = 0, sm1 = 0, sb0 = 0, sb1 = 0;  // select list ranges
};

struct HostStats {
  double runtime_run_ms = 0, runtime_divide_ms = 0, runtime_merge_ms = 0;
  double merge_prepare_ms = 0, merge_score_ms = 0, merge_select_ms = 0, merge_update_ms = 0;
  uint64_t iterations = 0, blocks = 0, groups_last = 0, active_last = 0;
  uint64_t compactions = 0;
  uint64_t divide_fallback_splits = 0;
};

// Timing of one kernel class with CUDA events on the engine stream.
enum TimedKernel : int { kTimeNone = 0, kTimeScore = 1, kTimePrepare = 2, kTimeUpdate = 3, kTimeDivide = 4 };

class Engine {
 public:
  Engine(int n, int64_t arcs, const int64_t* row_ptr, const int32_t* col_idx, const EngineConfig& cfg);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // Singleton partition rebuilt from the resident CSR (QuotientGraph::Initialize).
  void Reset();
  // Sweg::Run / Divide / Merge.
  void Run(int iterations);
  void Divide(int iter);
  void Merge(int iter, int total_iterations);

  // Scoring service: ExactMergeGainPersistent for arbitrary pairs of active reps.
  void ScorePairs(const int32_t* rep_a, const int32_t* rep_b, int64_t count, int64_t* gain, int64_t* before);
  // EA-proxy candidate generation for one explicit group of active reps.
  int64_t PrepareGroup(const int32_t* q, int g, int32_t* a_idx, int32_t* b_idx, int64_t cap);
  // Applies endpoint-disjoint merges (keep, remove) as one commit batch.
  void MergePairs(const int32_t* keep, const int32_t* remove, int64_t count);

  // Views of the state (host copies).
  void Partition(int32_t* labels, int32_t* head, int32_t* next);
  void Groups(int32_t* order, int32_t* starts, int32_t* lengths);
  int64_t ExportRow(int rep, int32_t* nb, int64_t* cnt, int64_t cap, int64_t* size, int64_t* internal);
  void DeviceStats(uint64_t* out, int count);
  int64_t QuotientNnz();
  // CostOracle::ExactPartitionCost of the current partition, from the input graph.
  int64_t ExactPartitionCost();
  // QuotientGraph::ValidateAgainstOriginalGraph: throws on the first mismatch.
  void ValidateQuotient();
  // Sweg::Encode of the current partition: P (supernode ids), Cp and Cm.
  void Encode(EncodeOutput* out);
  const HostStats& host_stats() const { return hstats_; }
  const RankerInfo& ranker_info() const { return rk_info_; }
  int64_t active_count() const { return n_active_; }
  int64_t group_count() const { return n_groups_; }
  int n() const { return n_; }
  int64_t arcs() const { return arcs_; }
  const EngineConfig& config() const { return cfg_; }
  cudaStream_t stream() const { return stream_; }

  // Kernel timing for the roofline: events around every launch of one kernel class.
  void SetTimedKernel(int which);
  double TimedKernelMs();
  int64_t TimedKernelLaunches() const { return timed_launches_; }
  void Synchronize();
  // Step timing with CUDA events on the engine stream.
  void StepTimerStart();
  double StepTimerStopMs();
  // Writes a buffer larger than the L2 cache on the engine stream.
  void FlushL2();
  // Number of this library's kernels launched since creation.
  int64_t launches() const { return launches_; }

 private:
  void CheckError();
  void InitQuotient();
  void EnsurePoolRoom();
  void EnsurePoolRoom(unsigned long long top);
  void CompactPool();
  void RunBlock(const BlockPlan& bp, double threshold, int iter, int total_iterations);
  void RankerReset();
  void RankerEnsure();
  void RankerLog(int rg0, int nrg, long long slots, int iter, double threshold, int total_iterations);
  void RankerRank(int rg0, int nrg, long long slots, double threshold, int iter);
  void RankerCutoff(long long slots);
  long long RankerExploreCap(long long slots) const;
  void RankerTrain();
  void RankerFinishIteration();
  void LaunchPrepare(const BlockPlan& bp);
  bool RowSumsOn(const BlockPlan& bp) const;
  void PlanOnDevice();
  void SizeIterationBuffers(size_t R, size_t ncand, size_t nsel, size_t nbig, long long max_mat, long long max_slots);
  void PrepareIterationBuffers();
  void BeginTimed(int which);
  void EndTimed(int which);
  void ConfigureKernels();
  QuotientView View();
  void LaunchCommit(int rg0, int nrg, int64_t max_pairs, bool verify);

  int n_;
  int64_t arcs_;
  EngineConfig cfg_;
  OwnedStream owned_stream_;
  cudaStream_t stream_ = nullptr;

  // graph
  DevBuf<long long> d_rowptr_;
  DevBuf<int> d_col_;
  DevBuf<int> d_arc_src_;

  // quotient graph
  DevBuf<Entry> d_pool_[2];
  int cur_pool_ = 0;
  size_t pool_cap_ = 0;
  DevBuf<unsigned long long> d_pool_top_;
  DevBuf<long long> d_qoff_;
  DevBuf<int> d_qlen_;
  DevBuf<int> d_qcap_;
  DevBuf<int> d_qsize_;
  DevBuf<long long> d_qint_;

  // partition
  DevBuf<int> d_label_, d_head_, d_next_, d_tail_, d_fwd_;
  DevBuf<int> d_stamp_, d_partner_, d_claim_, d_seq_;
  DevBuf<int> d_rows_short_, d_rows_long_;  // claimed neighbour rows of a block
  DevBuf<int> d_sel_list_;                   // selection slots of a block's selected pairs
  DevBuf<unsigned> d_rw_ticket_;             // last-CTA counter of the rewrite kernel

  // divide
  DevBuf<int> d_order_, d_head_flag_;
  DevBuf<unsigned long long> d_hash_, d_keys_, d_keys_alt_;
  DevBuf<int> d_vals_, d_vals_alt_;
  DevBuf<int> d_need_, d_seg_beg_, d_seg_end_, d_pos_map_;
  DevBuf<int> d_perm_, d_perm_alt_, d_segkey_, d_segkey_alt_;
  DevBuf<int> d_fix_list_;  // Divide: starts of equal-high-word runs with mixed low words
  DevBuf<unsigned> d_keys_hi_[2];  // Divide: high key words, the radix sort's keys
  DevBuf<unsigned long long> d_unf_pk_[2];  // Divide: packed unfinished-segment counts and their scan
  DevBuf<int> d_gstart_, d_glen_, d_group_of_, d_idx_in_group_;
  DevBuf<int> d_counts_;
  DevBuf<unsigned char> d_cub_tmp_;
  int need_stamp_ = 0;

  // per-iteration merge buffers
  DevBuf<long long> d_cand_off_, d_sel_off_, d_mat_off_;
  DevBuf<int2> d_cand_;
  DevBuf<int2> d_cand_rep_;  // per candidate slot: supernode ids (-1: unused)
  DevBuf<longlong2> d_res_;
  DevBuf<int> d_cand_cnt_;
  DevBuf<int> d_sel_keep_, d_sel_rem_;
  DevBuf<long long> d_sel_gain_;
  DevBuf<int> d_sel_cnt_;
  DevBuf<unsigned char> d_mat_;
  DevBuf<unsigned char> d_scratch_;
  DevBuf<BlockCtl> d_ctl_;
  DevBuf<unsigned long long> d_stats_;
  DevBuf<DevError> d_err_;
  std::vector<int> h_glen_;
  std::vector<unsigned> h_gent_;  // per group: row entries of its members at Divide time
  DevBuf<unsigned> d_gent_;
  std::vector<int> h_real_;      // Divide ids of the groups with >= 2 members
  std::vector<int> h_block_rg_;  // per 64-group block: first real-group position
  std::vector<int> h_small_, h_big_;              // real-group positions by prepare kernel
  std::vector<int> h_block_small_, h_block_big_;  // per block: first entry in those lists
  DevBuf<int> d_small_, d_big_;
  std::vector<int> h_sel_small_, h_sel_mid_, h_sel_big_;  // real-group positions by select kernel
  std::vector<int> h_block_sel_small_, h_block_sel_mid_, h_block_sel_big_;  // per block: first entries
  DevBuf<int> d_sel_small_, d_sel_mid_, d_sel_big_;
  DevBuf<unsigned char> d_bigdesc_;  // per big-group entry: deferred-group descriptor
  std::vector<long long> h_soff_;    // sort-slot prefix over h_big_ (deferred groups)
  DevBuf<long long> d_soff_;
  DevBuf<unsigned long long> d_skey_[2], d_sval_[2];
  std::vector<long long> h_big_moff_;  // member-count prefix over h_big_
  DevBuf<long long> d_big_moff_;
  DevBuf<int> d_real_;
  std::vector<long long> h_cand_off_, h_sel_off_, h_mat_off_;
  std::vector<BlockPlan> plans_;  // this iteration's blocks
  // per-row sums of a one-block iteration's block-start state (exact gain
  // from the shared neighbours only)
  DevBuf<long long> d_rc_before_, d_rc_light_;
  DevBuf<int4> d_rc_heavy_;
  DevBuf<int> d_rc_nheavy_;
  bool plan_on_device_ = false;
  int accum_grid_ = 152 * 4;  // resident CTAs of the dynamically scheduled kernels
  int score_grid_ = 152 * 4;   // one-block iteration: Merge plans it on the device
  DevBuf<unsigned char> d_plan_tiles_;
  DevBuf<long long> d_plan_scalars_;
  PinnedBuf<long long> h_pin_;
  int block_stamp_ = 0;
  int64_t n_active_ = 0;
  int64_t known_active_ = -1;  // active supernodes known on the host (-1: read it back)
  int64_t n_groups_ = 0;
  HostStats hstats_;

  // exact partition cost
  DevBuf<unsigned long long> d_pc_keys_[2], d_pc_scalars_;
  DevBuf<int> d_pc_counts_;

  // learned candidate ranker
  DevBuf<float2> d_cand_feat_;
  DevBuf<unsigned char> d_rk_keep_;
  DevBuf<float> d_rk_x_, d_rk_y_, d_rk_x2_, d_rk_y2_;  // training log, as appended / in (iteration, slot) order
  DevBuf<unsigned long long> d_rk_key_[2];
  DevBuf<int> d_rk_idx_[2];
  DevBuf<unsigned> d_rk_count_, d_rk_ticket_, d_rk_npos_;
  DevBuf<float> d_rk_params_, d_rk_m_, d_rk_v_, d_rk_norm_, d_rk_partial_, d_rk_loss_;
  DevBuf<unsigned short> d_rk_wbf_;
  DevBuf<double> d_rk_npartial_;
  DevBuf<float> d_rk_zbuf_, d_rk_zpos_[2], d_rk_cut_;  // per-slot logits, exploration positives, cutoff
  DevBuf<long long> d_rk_zgain_[2];                    // exact gains of the exploration positives
  bool rk_trained_ = false;
  float rk_cutoff_ = 0.0f;
  long long rk_iter_slots_ = 0;
  RankerInfo rk_info_;

  // launch accounting and step timing
  int64_t launches_ = 0;
  cudaEvent_t step_ev_[2] = {nullptr, nullptr};
  DevBuf<unsigned char> d_flush_;

  // kernel timing
  int timed_kind_ = kTimeNone;
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_used_ = 0;
  int64_t timed_launches_ = 0;
  double timed_ms_accum_ = 0.0;
};

}  // namespace beam
