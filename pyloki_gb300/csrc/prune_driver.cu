// One pruning level (prune.py:165-332 pruning_iteration_batched, Taylor and
// Chebyshev plugins on real folds) sequenced natively: branch, child count,
// resolve + shift-add + score, threshold selection (with the batch-sequential
// overflow rule when the survivors exceed the capacity) and emission of the
// new tree. The host waits twice per level, for the child count (to size the
// child arrays) and for the survivor count and score range, each read through
// the caller's pinned host words.
#include <algorithm>
#include <vector>

#include "loki_common.cuh"

using namespace loki;

extern "C" int loki_prune_level(const LokiPruneLevel* lvl, const LokiPruneTree* in,
                                LokiPruneTree* out, const LokiPruneWork* w,
                                const float* fold_segment, const LokiScoreSpec* spec,
                                double threshold, int64_t max_sugg, int64_t batch_size,
                                const uint8_t* parent_mask, LokiPruneLevelResult* res,
                                int32_t* dev_err, void* stream) {
  if (!lvl || !in || !out || !w || !fold_segment || !spec || !res || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (!w->host_words) return set_error(LOKI_ERR_INVALID, "host_words (pinned) is required");
  if (max_sugg < 1 || batch_size < 1) return set_error(LOKI_ERR_INVALID, "bad capacity");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t n_par = in->n;
  *res = LokiPruneLevelResult{};
  res->n_parents = n_par;
  if (n_par > w->par_cap) {
    res->need_par_cap = n_par;
    return set_error(LOKI_ERR_CAPACITY, "parent workspace holds %lld of %lld parents",
                     (long long)w->par_cap, (long long)n_par);
  }
  int rc = parent_mask
               ? loki_prune_branch_masked(lvl, in->leaves, n_par, parent_mask,
                                          (LokiBranchInfo*)w->info, w->offsets, w->scan,
                                          w->scan_bytes, dev_err, stream)
               : loki_prune_branch(lvl, in->leaves, n_par, (LokiBranchInfo*)w->info,
                                   w->offsets, w->scan, w->scan_bytes, dev_err, stream);
  if (rc) return rc;
  // wait 1: child count and the error word
  int64_t* hw = w->host_words;
  if (cudaMemcpyAsync(hw, w->offsets + n_par, sizeof(int64_t), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(hw + 1, dev_err, sizeof(int32_t), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "reading the child count failed");
  const int64_t n_child = hw[0];
  res->n_children = n_child;
  if (*reinterpret_cast<int32_t*>(hw + 1) != 0) {
    res->dev_err = *reinterpret_cast<int32_t*>(hw + 1);
    return LOKI_OK;  // the caller decodes the error word (branch_max)
  }
  if (n_child > w->child_cap) {
    res->need_child_cap = n_child;
    return set_error(LOKI_ERR_CAPACITY, "child workspace holds %lld of %lld children",
                     (long long)w->child_cap, (long long)n_child);
  }
  if (w->ev_score_begin) cudaEventRecord((cudaEvent_t)w->ev_score_begin, s);
  rc = loki_prune_score(lvl, in->leaves, in->folds, n_par, (const LokiBranchInfo*)w->info,
                        w->offsets, n_child, fold_segment, spec, w->child_scores,
                        w->child_idx, w->child_phase, w->minmax, dev_err, stream);
  if (rc) return rc;
  if (w->ev_score_end) cudaEventRecord((cudaEvent_t)w->ev_score_end, s);
  rc = loki_prune_select(w->child_scores, n_child, threshold, w->surv, w->n_surv, w->sscan,
                         w->sscan_bytes, stream);
  if (rc) return rc;
  // wait 2: survivor count and score range
  if (cudaMemcpyAsync(hw + 2, w->n_surv, sizeof(int64_t), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      (n_child &&
       cudaMemcpyAsync(hw + 3, w->minmax, 2 * sizeof(float), cudaMemcpyDeviceToHost, s) !=
           cudaSuccess) ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "reading the survivor count failed");
  int64_t n_surv = hw[2];
  if (n_child) {
    const float* mm = reinterpret_cast<const float*>(hw + 3);
    res->score_min = mm[0];
    res->score_max = mm[1];
  }
  if (n_surv > max_sugg) {
    // the reference's batch-sequential overflow rule: scratch sized by the
    // largest parent batch's children
    std::vector<int64_t> off(n_par + 1);
    if (cudaMemcpy(off.data(), w->offsets, (n_par + 1) * sizeof(int64_t),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "reading the offsets failed");
    int64_t max_batch = 0;
    for (int64_t b0 = 0; b0 < n_par; b0 += batch_size)
      max_batch = std::max(max_batch, off[std::min(b0 + batch_size, n_par)] - off[b0]);
    const int64_t need = max_sugg + max_batch + 1;
    if (need > w->ovf_cap) {
      res->need_ovf_cap = need;
      return set_error(LOKI_ERR_CAPACITY, "overflow scratch holds %lld of %lld",
                       (long long)w->ovf_cap, (long long)need);
    }
    rc = loki_prune_select_overflow(w->child_scores, w->offsets, n_par, batch_size, threshold,
                                    max_sugg, w->surv, w->n_surv, w->ovf_thr, w->ovf_ids,
                                    w->ovf_keys, need, stream);
    if (rc) return rc;
    if (cudaMemcpyAsync(hw + 2, w->n_surv, sizeof(int64_t), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "reading the survivor count failed");
    n_surv = hw[2];
    res->overflow = 1;
  }
  res->n_surv = n_surv;
  if (n_surv > out->cap) {
    res->need_tree_cap = n_surv;
    return set_error(LOKI_ERR_CAPACITY, "output tree holds %lld of %lld leaves",
                     (long long)out->cap, (long long)n_surv);
  }
  out->n = n_surv;
  if (n_surv == 0) return LOKI_OK;
  return loki_prune_emit(lvl, in->leaves, in->folds, (const LokiBranchInfo*)w->info,
                         w->offsets, n_par, fold_segment, w->surv, n_surv, w->child_scores,
                         w->child_idx, w->child_phase, out->leaves, out->folds, out->scores,
                         out->scores_ep, out->backtracks, stream);
}
