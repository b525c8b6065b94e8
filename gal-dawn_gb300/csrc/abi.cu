// extern "C" entry points of libdawn_gb300.so (declared in include/dawn_gb300.h).
//
// Argument checking, graph upload, staging of host buffers and statistics
// live here; the traversals themselves are in bovm.cu (single-source
// expand), msbfs.cu (64-source bitset expand) and govm.cu (min-plus relax).
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "dawn_internal.cuh"
#include "selector_default.inc"

using dawn::DevBuf;

namespace dawn {

// Whether this call's decide kernels evaluate the selector, and with which
// weights in the handle's slot: the handle's own (dawn_graph_set_selector),
// else for DAWN_VARIANT_LEARNED the library's trained defaults, else none
// (direction heuristics).
dawn_status call_selector(dawn_graph* g, int32_t variant, int32_t* use) {
  *use = 0;
  int want = g->sel_on ? 1 : 0;
#if DAWN_HAVE_DEFAULT_SELECTOR
  static_assert(sizeof(kDefaultSelectorWeights) == sizeof(float) * DAWN_SELECTOR_WEIGHTS,
                "default selector weight count");
  if (!want && variant == DAWN_VARIANT_LEARNED) want = 2;
#else
  (void)variant;
#endif
  if (!want) return DAWN_OK;
  if (g->sel_slot_state != want) {
#if DAWN_HAVE_DEFAULT_SELECTOR
    const float* src = want == 1 ? g->sel_user.data() : kDefaultSelectorWeights;
#else
    const float* src = g->sel_user.data();
#endif
    DAWN_CUDA(cudaMemcpyAsync(g->sel_slot.p, src, sizeof(float) * DAWN_SELECTOR_WEIGHTS, cudaMemcpyHostToDevice,
                              g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    g->sel_slot_state = want;
  }
  *use = 1;
  return DAWN_OK;
}

void drop_graphs(dawn_graph* g) {
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->bfs_exec) cudaGraphExecDestroy(g->bfs_exec);
  if (g->sssp_exec) cudaGraphExecDestroy(g->sssp_exec);
  if (g->mw_exec) cudaGraphExecDestroy(g->mw_exec);
  g->bfs_exec = g->sssp_exec = g->mw_exec = nullptr;
  for (cudaGraphExec_t& e : g->bs_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
}

}  // namespace dawn

namespace {

constexpr size_t kStageBytes = (size_t)1 << 31;  // host-pointer calls: device staging per chunk

dawn_status check_sources(const dawn_graph* g, const int32_t* sources, int32_t nsrc) {
  if (nsrc < 0 || (nsrc > 0 && !sources)) {
    dawn::set_error("invalid source list (nsrc = %d)", nsrc);
    return DAWN_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < nsrc; i++)
    if (sources[i] < 0 || sources[i] >= g->n) {
      dawn::set_error("source %d (index %d) outside [0, %d)", sources[i], i, g->n);
      return DAWN_ERR_INVALID_ARG;
    }
  return DAWN_OK;
}

dawn_status finish_graph(dawn_graph* g, uint32_t flags) {
  if (!(flags & DAWN_GRAPH_NO_VALIDATE)) DAWN_CHECK(dawn::validate_csr(g));
  if (g->symmetric) {
    g->t_row_ptr = g->row_ptr;
    g->t_col = g->col;
  } else {
    DAWN_CHECK(dawn::build_transpose(g));
  }
  static_assert(2 * sizeof(dawn::SsCtl) <= dawn::kPinnedSlot, "control-block copies exceed a pinned slot");
  DAWN_CHECK(dawn::pinned_slot((void**)&g->h_ctl));
  DAWN_CHECK(dawn::ensure(g->sel_slot, sizeof(float) * DAWN_SELECTOR_WEIGHTS, g->stream));
  DAWN_CUDA(cudaEventCreate(&g->ev0));
  DAWN_CUDA(cudaEventCreate(&g->ev1));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

dawn_status start_graph(dawn_wtype wtype, int32_t n, int64_t m, uint32_t flags, void* stream, dawn_graph** out,
                        const void* row_ptr, const void* col, const void* val, dawn_graph** gp) {
  if (!out) {
    dawn::set_error("out is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (n < 1 || m < 0 || m > INT32_MAX || !row_ptr || (m > 0 && !col) ||
      (wtype != DAWN_W_NONE && wtype != DAWN_W_I32 && wtype != DAWN_W_F32) ||
      (wtype != DAWN_W_NONE && m > 0 && !val)) {
    dawn::set_error("invalid graph arguments (n = %d, m = %lld, wtype = %d)", n, (long long)m, (int)wtype);
    return DAWN_ERR_INVALID_ARG;
  }
  dawn_graph* g = new dawn_graph();
  *gp = g;
  g->n = n;
  g->m = m;
  g->flags = flags;
  g->wtype = wtype;
  g->symmetric = (flags & DAWN_GRAPH_SYMMETRIC) != 0;
  DAWN_CUDA(cudaGetDevice(&g->device));
  DAWN_CUDA(cudaDeviceGetAttribute(&g->geo.sms, cudaDevAttrMultiProcessorCount, g->device));
  if (stream) {
    g->stream = static_cast<cudaStream_t>(stream);
  } else {
    DAWN_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    g->own_stream = true;
  }
  // col / val carry 32 spare bytes so 256-bit loads at a row's end stay in bounds.
  DAWN_CHECK(dawn::pool_alloc((void**)&g->row_ptr, sizeof(int32_t) * ((size_t)n + 1), g->stream));
  DAWN_CHECK(dawn::pool_alloc((void**)&g->col, sizeof(int32_t) * (size_t)(m > 0 ? m : 1) + 32, g->stream));
  if (wtype != DAWN_W_NONE)
    DAWN_CHECK(dawn::pool_alloc(&g->val, sizeof(int32_t) * (size_t)(m > 0 ? m : 1) + 32, g->stream));
  return DAWN_OK;
}

void destroy(dawn_graph* g) {
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->t_row_ptr && g->t_row_ptr != g->row_ptr) dawn::pool_free(g->t_row_ptr, g->stream);
  if (g->t_col && g->t_col != g->col) dawn::pool_free(g->t_col, g->stream);
  dawn::pool_free(g->row_ptr, g->stream);
  dawn::pool_free(g->col, g->stream);
  if (g->val) dawn::pool_free(g->val, g->stream);
  DevBuf* bufs[] = {&g->ss_queues, &g->ss_segs, &g->bs_segs, &g->ss_bitmaps, &g->ss_ctl, &g->ss_sources, &g->ss_scratch,
                    &g->bs_words, &g->bs_queues, &g->bs_ctl, &g->bs_sources, &g->ul_static, &g->hv_static, &g->hv_segoff, &g->hv_acc, &g->hv_tasks, &g->cc_out,
                    &g->dist_stage, &g->pt_voff, &g->pt_tasks, &g->pt_sources, &g->pt_ctl, &g->pt_scratch, &g->pt_rows,
                    &g->sel_slot, &g->wt_col, &g->wt_val, &g->mw_block, &g->mw_masks,
                    &g->mw_ctl, &g->mw_sources, &g->bc_levels, &g->bc_terms, &g->bc_range, &g->bc_out,
                    &g->bc_heavy, &g->bc_part};
  for (DevBuf* b : bufs) dawn::release(*b);
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->bfs_exec) cudaGraphExecDestroy(g->bfs_exec);
  if (g->sssp_exec) cudaGraphExecDestroy(g->sssp_exec);
  for (cudaGraphExec_t e : g->bs_exec)
    if (e) cudaGraphExecDestroy(e);
  if (g->pt_exec) cudaGraphExecDestroy(g->pt_exec);
  if (g->mw_exec) cudaGraphExecDestroy(g->mw_exec);
  dawn::pinned_slot_release(g->h_ctl);
  dawn::pinned_slot_release(g->bc_h_level);
  for (cudaEvent_t e : g->trace_ev)
    if (e) cudaEventDestroy(e);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

int32_t resolve_variant(const dawn_graph* g, int32_t variant, int32_t nsrc) {
  if (variant == DAWN_VARIANT_AUTO)
    return nsrc >= 2 ? (g->auto_learned ? DAWN_VARIANT_LEARNED : DAWN_VARIANT_BITSET) : DAWN_VARIANT_DO;
  return variant;
}

dawn_status bfs_device_impl(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist,
                            int32_t variant, dawn_stats* st) {
  variant = resolve_variant(g, variant, nsrc);
  DAWN_CHECK(dawn::call_selector(g, variant, &g->sel_call));
  if (st) {
    std::memset(st, 0, sizeof(*st));
    DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
  }
  if (variant == DAWN_VARIANT_PUSH || variant == DAWN_VARIANT_DO) {
    DAWN_CHECK(dawn::bfs_single(g, sources, nsrc, d_dist, variant));
    if (st) {
      DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
      dawn::SsCtl c;
      DAWN_CHECK(dawn::download_ctl(g, &c));
      st->edges_traversed = (int64_t)c.total_reached;
      st->levels = c.total_levels;
      st->push_levels = c.total_push;
      st->pull_levels = c.total_pull;
      st->batches = nsrc;
    }
  } else if (variant == DAWN_VARIANT_BITSET || variant == DAWN_VARIANT_LEARNED) {
    DAWN_CHECK(dawn::bfs_bitset(g, sources, nsrc, d_dist));
    if (st) {
      DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
      DAWN_CHECK(dawn::bfs_bitset_stats(g, st, nsrc));
    }
  } else {
    dawn::set_error("unknown BFS variant %d", variant);
    return DAWN_ERR_UNSUPPORTED;
  }
  if (st) {
    DAWN_CUDA(cudaEventSynchronize(g->ev1));
    DAWN_CUDA(cudaEventElapsedTime(&st->device_ms, g->ev0, g->ev1));
  }
  return DAWN_OK;
}

// Batched (64 sources per traversal) unless the caller asks for the
// single-source kernels or there is one source.
bool sssp_uses_batch(int32_t variant, int32_t nsrc) {
  return nsrc >= 2 && variant != DAWN_VARIANT_PUSH && variant != DAWN_VARIANT_DO;
}

dawn_status sssp_device_impl(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* d_dist,
                             dawn_stats* st, int32_t variant = DAWN_VARIANT_AUTO) {
  if (st) {
    std::memset(st, 0, sizeof(*st));
    DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
  }
  if (sssp_uses_batch(variant, nsrc)) {
    DAWN_CHECK(dawn::sssp_batched(g, sources, nsrc, d_dist));
    if (st) {
      DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
      DAWN_CHECK(dawn::sssp_batched_stats(g, st, nsrc));
      DAWN_CUDA(cudaEventElapsedTime(&st->device_ms, g->ev0, g->ev1));
    }
    return DAWN_OK;
  }
  DAWN_CHECK(dawn::sssp_single(g, sources, nsrc, d_dist));
  if (st) {
    DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
    dawn::SsCtl c;
    DAWN_CHECK(dawn::download_ctl(g, &c));
    st->levels = c.total_levels;
    st->push_levels = c.total_push;
    st->pull_levels = c.total_pull;
    st->batches = nsrc;
    DAWN_CUDA(cudaEventElapsedTime(&st->device_ms, g->ev0, g->ev1));
    // TEPS numerator: out-degree sum of the reached vertices of every row.
    DAWN_CHECK(dawn::ensure(g->cc_out, 16 * (size_t)nsrc, g->stream));
    double* sum = g->cc_out.as<double>();
    long long* cnt = reinterpret_cast<long long*>(sum + nsrc);
    DAWN_CHECK(dawn::row_reduce(g, d_dist, nsrc, g->ss_sources.as<int32_t>(), g->wtype == DAWN_W_F32 ? 2 : 1,
                                1, sum, cnt));
    std::vector<long long> h(nsrc);
    DAWN_CUDA(cudaMemcpyAsync(h.data(), sum, sizeof(long long) * nsrc, cudaMemcpyDeviceToHost, g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    for (long long x : h) st->edges_traversed += x;
  }
  return DAWN_OK;
}

void add_stats(dawn_stats* acc, const dawn_stats& s) {
  acc->edges_traversed += s.edges_traversed;
  acc->levels += s.levels;
  acc->push_levels += s.push_levels;
  acc->pull_levels += s.pull_levels;
  acc->batches += s.batches;
  acc->device_ms += s.device_ms;
}

// Runs a device traversal in chunks of sources through device staging and
// copies each chunk's rows to the caller's host array.
bool is_pinned_host(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

template <class Fn>
dawn_status staged(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* host_dist, size_t elem,
                   dawn_stats* st, Fn&& run, bool direct_ok = false) {
  const size_t row_bytes = elem * (size_t)g->n;
  if (direct_ok && is_pinned_host(host_dist)) {
    // The traversal writes its distances only in its final pass, so the
    // caller's page-locked buffer can take them directly over the host
    // link: no device staging and no separate copy.
    DAWN_CHECK(run(sources, nsrc, host_dist, st));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    return DAWN_OK;
  }
  int32_t chunk = (int32_t)(kStageBytes / row_bytes);
  if (chunk >= 64) chunk -= chunk % 64;
  if (chunk < 1) chunk = 1;
  if (chunk > nsrc) chunk = nsrc;
  DAWN_CHECK(dawn::ensure(g->dist_stage, row_bytes * (size_t)chunk, g->stream));
  if (st) std::memset(st, 0, sizeof(*st));
  for (int32_t i0 = 0; i0 < nsrc; i0 += chunk) {
    const int32_t c = nsrc - i0 < chunk ? nsrc - i0 : chunk;
    dawn_stats s;
    DAWN_CHECK(run(sources + i0, c, g->dist_stage.p, st ? &s : nullptr));
    if (host_dist)
      DAWN_CUDA(cudaMemcpyAsync(static_cast<char*>(host_dist) + row_bytes * (size_t)i0, g->dist_stage.p,
                                row_bytes * (size_t)c, cudaMemcpyDeviceToHost, g->stream));
    if (st) add_stats(st, s);
  }
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

long long multi_out_elems(const dawn_graph* g, const int32_t* source_offset) {
  long long out = 0;
  const int32_t nparts = (int32_t)g->pt_off.size() - 1;
  for (int32_t p = 0; p < nparts; p++)
    out += (long long)(source_offset[p + 1] - source_offset[p]) * (g->pt_off[p + 1] - g->pt_off[p]);
  return out;
}

dawn_status multi_args(const dawn_graph* g, const int32_t* source_offset, const int32_t* sources) {
  if (!g || !source_offset) {
    dawn::set_error("graph or source_offset is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (g->pt_off.size() < 2) {
    dawn::set_error("the graph has no parts: call dawn_graph_set_parts first");
    return DAWN_ERR_INVALID_ARG;
  }
  const int32_t nparts = (int32_t)g->pt_off.size() - 1;
  if (source_offset[0] != 0) {
    dawn::set_error("source_offset[0] must be 0");
    return DAWN_ERR_INVALID_ARG;
  }
  for (int32_t p = 0; p < nparts; p++)
    if (source_offset[p + 1] < source_offset[p]) {
      dawn::set_error("source_offset decreases at part %d", p);
      return DAWN_ERR_INVALID_ARG;
    }
  if (source_offset[nparts] > 0 && !sources) {
    dawn::set_error("sources is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  return DAWN_OK;
}

}  // namespace

extern "C" {

const char* dawn_last_error(void) { return dawn::last_error(); }

const char* dawn_version(void) { return "dawn_gb300 0.1 (sm_103a)"; }

dawn_status dawn_graph_create(const int32_t* row_ptr, const int32_t* col, const void* val, dawn_wtype wtype,
                              int32_t n, int64_t m, uint32_t flags, void* stream, dawn_graph** out) {
  dawn::clear_error();
  dawn_graph* g = nullptr;
  dawn_status s = start_graph(wtype, n, m, flags, stream, out, row_ptr, col, val, &g);
  if (s == DAWN_OK) {
    do {
      cudaError_t e = cudaMemcpyAsync(g->row_ptr, row_ptr, sizeof(int32_t) * ((size_t)n + 1),
                                      cudaMemcpyHostToDevice, g->stream);
      if (e == cudaSuccess && m > 0)
        e = cudaMemcpyAsync(g->col, col, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, g->stream);
      if (e == cudaSuccess && m > 0 && g->val)
        e = cudaMemcpyAsync(g->val, val, sizeof(int32_t) * (size_t)m, cudaMemcpyHostToDevice, g->stream);
      if (e != cudaSuccess) {
        dawn::set_error("CSR upload: %s", cudaGetErrorString(e));
        s = DAWN_ERR_CUDA;
        break;
      }
      s = finish_graph(g, flags);
    } while (0);
  }
  if (s != DAWN_OK) {
    destroy(g);
    return s;
  }
  *out = g;
  return DAWN_OK;
}

dawn_status dawn_graph_create_device(const int32_t* d_row_ptr, const int32_t* d_col, const void* d_val,
                                     dawn_wtype wtype, int32_t n, int64_t m, uint32_t flags, void* stream,
                                     dawn_graph** out) {
  dawn::clear_error();
  dawn_graph* g = nullptr;
  dawn_status s = start_graph(wtype, n, m, flags, stream, out, d_row_ptr, d_col, d_val, &g);
  if (s == DAWN_OK) {
    do {
      cudaError_t e = cudaMemcpyAsync(g->row_ptr, d_row_ptr, sizeof(int32_t) * ((size_t)n + 1),
                                      cudaMemcpyDeviceToDevice, g->stream);
      if (e == cudaSuccess && m > 0)
        e = cudaMemcpyAsync(g->col, d_col, sizeof(int32_t) * (size_t)m, cudaMemcpyDeviceToDevice, g->stream);
      if (e == cudaSuccess && m > 0 && g->val)
        e = cudaMemcpyAsync(g->val, d_val, sizeof(int32_t) * (size_t)m, cudaMemcpyDeviceToDevice, g->stream);
      if (e != cudaSuccess) {
        dawn::set_error("CSR copy: %s", cudaGetErrorString(e));
        s = DAWN_ERR_CUDA;
        break;
      }
      s = finish_graph(g, flags);
    } while (0);
  }
  if (s != DAWN_OK) {
    destroy(g);
    return s;
  }
  *out = g;
  return DAWN_OK;
}

dawn_status dawn_graph_destroy(dawn_graph* g) {
  dawn::clear_error();
  destroy(g);
  return DAWN_OK;
}

dawn_status dawn_graph_set_stream(dawn_graph* g, void* stream) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  if (g->own_stream) cudaStreamDestroy(g->stream);
  g->own_stream = false;
  if (stream) {
    g->stream = static_cast<cudaStream_t>(stream);
  } else {
    DAWN_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    g->own_stream = true;
  }
  return DAWN_OK;
}

dawn_status dawn_graph_synchronize(dawn_graph* g) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

dawn_status dawn_bfs_device(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* d_dist,
                            int32_t variant, dawn_stats* stats) {
  dawn::clear_error();
  if (!g || (nsrc > 0 && !d_dist)) {
    dawn::set_error("graph or distance buffer is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (nsrc == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return DAWN_OK;
  }
  return bfs_device_impl(g, sources, nsrc, d_dist, variant, stats);
}

dawn_status dawn_bfs(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t* dist, int32_t variant,
                     dawn_stats* stats) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (nsrc == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return DAWN_OK;
  }
  const int32_t v = resolve_variant(g, variant, nsrc);
  return staged(
      g, sources, nsrc, dist, sizeof(int32_t), stats,
      [&](const int32_t* s, int32_t c, void* d, dawn_stats* st) {
        return bfs_device_impl(g, s, c, static_cast<int32_t*>(d), variant, st);
      },
      v == DAWN_VARIANT_BITSET || v == DAWN_VARIANT_LEARNED);
}

dawn_status dawn_sssp_device(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* d_dist, int32_t variant,
                             dawn_stats* stats) {
  dawn::clear_error();
  if (!g || (nsrc > 0 && !d_dist)) {
    dawn::set_error("graph or distance buffer is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (g->wtype == DAWN_W_NONE) {
    dawn::set_error("dawn_sssp needs a weighted graph");
    return DAWN_ERR_UNSUPPORTED;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (nsrc == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return DAWN_OK;
  }
  return sssp_device_impl(g, sources, nsrc, d_dist, stats, variant);
}

dawn_status dawn_sssp(dawn_graph* g, const int32_t* sources, int32_t nsrc, void* dist, int32_t variant,
                      dawn_stats* stats) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (g->wtype == DAWN_W_NONE) {
    dawn::set_error("dawn_sssp needs a weighted graph");
    return DAWN_ERR_UNSUPPORTED;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (nsrc == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return DAWN_OK;
  }
  return staged(
      g, sources, nsrc, dist, sizeof(int32_t), stats,
      [&](const int32_t* s, int32_t c, void* d, dawn_stats* st) { return sssp_device_impl(g, s, c, d, st, variant); },
      sssp_uses_batch(variant, nsrc));
}

dawn_status dawn_closeness(dawn_graph* g, const int32_t* sources, int32_t nsrc, int32_t weighted, double* cc,
                           double* dist_sum, int64_t* reached, dawn_stats* stats) {
  dawn::clear_error();
  if (!g || (nsrc > 0 && !cc)) {
    dawn::set_error("graph or output is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (weighted && g->wtype == DAWN_W_NONE) {
    dawn::set_error("weighted closeness needs a weighted graph");
    return DAWN_ERR_UNSUPPORTED;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (nsrc == 0) return DAWN_OK;
  const int kind = !weighted ? 0 : (g->wtype == DAWN_W_F32 ? 2 : 1);
  if (kind == 0) {
    // Hop closeness straight from the batched traversal's level words: its
    // final pass sums each source's distances instead of writing them, so
    // no distance matrix is formed.
    DAWN_CHECK(dawn::ensure(g->cc_out, 2 * sizeof(unsigned long long) * (size_t)nsrc, g->stream));
    unsigned long long* d_sum = g->cc_out.as<unsigned long long>();
    unsigned long long* d_cnt = d_sum + nsrc;
    DAWN_CUDA(cudaMemsetAsync(d_sum, 0, 2 * sizeof(unsigned long long) * (size_t)nsrc, g->stream));
    DAWN_CHECK(dawn::call_selector(g, DAWN_VARIANT_BITSET, &g->sel_call));
    if (stats) DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
    DAWN_CHECK(dawn::bfs_bitset(g, sources, nsrc, nullptr, d_sum, d_cnt));
    if (stats) {
      DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
      DAWN_CHECK(dawn::bfs_bitset_stats(g, stats, nsrc));
      DAWN_CUDA(cudaEventSynchronize(g->ev1));
      DAWN_CUDA(cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1));
    }
    std::vector<unsigned long long> h(2 * (size_t)nsrc);
    DAWN_CUDA(cudaMemcpyAsync(h.data(), d_sum, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                              g->stream));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    for (int32_t i = 0; i < nsrc; i++) {
      const double total = (double)h[i];
      cc[i] = total > 0 ? (double)(g->n - 1) / total : 0.0;
      if (dist_sum) dist_sum[i] = total;
      // the count includes the source's own bit (level 0)
      if (reached) reached[i] = (int64_t)h[nsrc + i] - 1;
    }
    return DAWN_OK;
  }
  const size_t row_bytes = sizeof(int32_t) * (size_t)g->n;
  int32_t chunk = (int32_t)(kStageBytes / row_bytes);
  if (chunk >= 64) chunk -= chunk % 64;
  if (chunk < 1) chunk = 1;
  if (chunk > nsrc) chunk = nsrc;
  DAWN_CHECK(dawn::ensure(g->dist_stage, row_bytes * (size_t)chunk, g->stream));
  DAWN_CHECK(dawn::ensure(g->cc_out, 16 * (size_t)chunk, g->stream));
  DevBuf srcbuf;
  DAWN_CHECK(dawn::ensure(srcbuf, sizeof(int32_t) * (size_t)chunk, g->stream));
  std::vector<double> hsum(chunk);
  std::vector<long long> hcnt(chunk);
  dawn_status s = DAWN_OK;
  for (int32_t i0 = 0; i0 < nsrc && s == DAWN_OK; i0 += chunk) {
    const int32_t c = nsrc - i0 < chunk ? nsrc - i0 : chunk;
    dawn_stats one;
    if (weighted)
      s = sssp_device_impl(g, sources + i0, c, g->dist_stage.p, stats ? &one : nullptr);
    else
      s = bfs_device_impl(g, sources + i0, c, g->dist_stage.as<int32_t>(), DAWN_VARIANT_AUTO,
                          stats ? &one : nullptr);
    if (s != DAWN_OK) break;
    if (stats) add_stats(stats, one);
    double* sum = g->cc_out.as<double>();
    long long* cnt = reinterpret_cast<long long*>(sum + chunk);
    if (cudaMemcpyAsync(srcbuf.p, sources + i0, sizeof(int32_t) * c, cudaMemcpyHostToDevice, g->stream) !=
        cudaSuccess) {
      dawn::set_error("source upload failed");
      s = DAWN_ERR_CUDA;
      break;
    }
    if ((s = dawn::row_reduce(g, g->dist_stage.p, c, srcbuf.as<int32_t>(), kind, 0, sum, cnt)) != DAWN_OK) break;
    if (cudaMemcpyAsync(hsum.data(), sum, sizeof(double) * c, cudaMemcpyDeviceToHost, g->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(hcnt.data(), cnt, sizeof(long long) * c, cudaMemcpyDeviceToHost, g->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(g->stream) != cudaSuccess) {
      dawn::set_error("closeness read-back failed");
      s = DAWN_ERR_CUDA;
      break;
    }
    for (int32_t i = 0; i < c; i++) {
      double total;
      if (kind == 2) {
        total = hsum[i];
      } else {
        long long bits;
        std::memcpy(&bits, &hsum[i], sizeof(bits));
        total = (double)bits;
      }
      cc[i0 + i] = total > 0 ? (double)(g->n - 1) / total : 0.0;
      if (dist_sum) dist_sum[i0 + i] = total;
      if (reached) reached[i0 + i] = hcnt[i];
    }
  }
  dawn::release(srcbuf);
  return s;
}

dawn_status dawn_betweenness_device(dawn_graph* g, const int32_t* sources, int32_t nsrc, double* d_bc,
                                    dawn_stats* stats) {
  dawn::clear_error();
  if (!g || !d_bc) {
    dawn::set_error("graph or output is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  if (stats) DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
  DAWN_CHECK(dawn::betweenness(g, sources, nsrc, d_bc, stats));
  if (stats) {
    DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
    DAWN_CUDA(cudaEventSynchronize(g->ev1));
    DAWN_CUDA(cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1));
  }
  return DAWN_OK;
}

dawn_status dawn_betweenness(dawn_graph* g, const int32_t* sources, int32_t nsrc, double* bc, dawn_stats* stats) {
  dawn::clear_error();
  if (!g || !bc) {
    dawn::set_error("graph or output is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(dawn::ensure(g->bc_out, sizeof(double) * (size_t)g->n, g->stream));
  DAWN_CHECK(dawn_betweenness_device(g, sources, nsrc, g->bc_out.as<double>(), stats));
  DAWN_CUDA(cudaMemcpyAsync(bc, g->bc_out.p, sizeof(double) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

dawn_status dawn_graph_set_parts(dawn_graph* g, int32_t nparts, const int32_t* offsets) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  return dawn::parts_set(g, nparts, offsets);
}

dawn_status dawn_multi_bfs_device(dawn_graph* g, const int32_t* source_offset, const int32_t* sources,
                                  int32_t* d_dist, dawn_stats* stats) {
  dawn::clear_error();
  DAWN_CHECK(multi_args(g, source_offset, sources));
  if (!d_dist && multi_out_elems(g, source_offset) > 0) {
    dawn::set_error("dist is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (stats) DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
  DAWN_CHECK(dawn::parts_bfs(g, source_offset, sources, d_dist, nullptr, stats));
  if (stats) {
    DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
    DAWN_CUDA(cudaEventSynchronize(g->ev1));
    DAWN_CUDA(cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1));
  }
  return DAWN_OK;
}

dawn_status dawn_multi_bfs(dawn_graph* g, const int32_t* source_offset, const int32_t* sources, int32_t* dist,
                           dawn_stats* stats) {
  dawn::clear_error();
  DAWN_CHECK(multi_args(g, source_offset, sources));
  const long long elems = multi_out_elems(g, source_offset);
  if (!dist && elems > 0) {
    dawn::set_error("dist is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (elems == 0) return dawn_multi_bfs_device(g, source_offset, sources, nullptr, stats);
  if (is_pinned_host(dist)) {
    // distances are written once, by the final pass of each task: a
    // page-locked buffer takes them directly
    DAWN_CHECK(dawn_multi_bfs_device(g, source_offset, sources, dist, stats));
    DAWN_CUDA(cudaStreamSynchronize(g->stream));
    return DAWN_OK;
  }
  const size_t bytes = sizeof(int32_t) * (size_t)elems;
  DAWN_CHECK(dawn::ensure(g->dist_stage, bytes, g->stream));
  DAWN_CHECK(dawn_multi_bfs_device(g, source_offset, sources, g->dist_stage.as<int32_t>(), stats));
  DAWN_CUDA(cudaMemcpyAsync(dist, g->dist_stage.p, bytes, cudaMemcpyDeviceToHost, g->stream));
  DAWN_CUDA(cudaStreamSynchronize(g->stream));
  return DAWN_OK;
}

dawn_status dawn_multi_closeness(dawn_graph* g, const int32_t* source_offset, const int32_t* sources, double* cc,
                                 double* dist_sum, int64_t* reached, dawn_stats* stats) {
  dawn::clear_error();
  DAWN_CHECK(multi_args(g, source_offset, sources));
  const int32_t nparts = (int32_t)g->pt_off.size() - 1;
  const int32_t nsrc = source_offset[nparts];
  if (nsrc > 0 && !cc) {
    dawn::set_error("cc is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  const long long elems = multi_out_elems(g, source_offset);
  if (elems == 0) return dawn_multi_bfs_device(g, source_offset, sources, nullptr, stats);
  DAWN_CHECK(dawn::ensure(g->dist_stage, sizeof(int32_t) * (size_t)elems, g->stream));
  std::vector<dawn::PartRow> rows;
  if (stats) DAWN_CUDA(cudaEventRecord(g->ev0, g->stream));
  DAWN_CHECK(dawn::parts_bfs(g, source_offset, sources, g->dist_stage.as<int32_t>(), &rows, stats));
  std::vector<long long> hs(rows.size()), hc(rows.size());
  DAWN_CHECK(dawn::parts_row_reduce(g, g->dist_stage.as<int32_t>(), rows, hs.data(), hc.data()));
  if (stats) {
    DAWN_CUDA(cudaEventRecord(g->ev1, g->stream));
    DAWN_CUDA(cudaEventSynchronize(g->ev1));
    DAWN_CUDA(cudaEventElapsedTime(&stats->device_ms, g->ev0, g->ev1));
  }
  for (size_t i = 0; i < rows.size(); i++) {
    const double total = (double)hs[i];
    cc[i] = total > 0 ? (double)(rows[i].len - 1) / total : 0.0;
    if (dist_sum) dist_sum[i] = total;
    if (reached) reached[i] = hc[i];
  }
  return DAWN_OK;
}

dawn_status dawn_bfs_static(const int32_t* row_ptr, const int32_t* col, int32_t n, int64_t m, int32_t source,
                            int32_t* dist, uint32_t flags, void* stream) {
  dawn::clear_error();
  return dawn::bfs_static(row_ptr, col, n, m, source, dist, flags, static_cast<cudaStream_t>(stream));
}

dawn_status dawn_graph_set_option(dawn_graph* g, int32_t option, int64_t value) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  switch (option) {
    case DAWN_OPT_BITSET_WIDTH:
      if (value != 0 && value != 1 && value != 2 && value != 4) {
        dawn::set_error("bitset width must be 0 (automatic), 1, 2 or 4");
        return DAWN_ERR_INVALID_ARG;
      }
      g->bs_width = (int32_t)value;
      return DAWN_OK;
    case DAWN_OPT_PUSH_RATIO:
      if (value < 1 || value > 1 << 20) {
        dawn::set_error("push ratio must lie in [1, 2^20]");
        return DAWN_ERR_INVALID_ARG;
      }
      g->bs_push_ratio = (int32_t)value;
      return DAWN_OK;
    case DAWN_OPT_FORCE_VARIANT:
      if (value < 0 || value > 3) {
        dawn::set_error("forced variant must be 0 (decide per level), 1, 2 or 3");
        return DAWN_ERR_INVALID_ARG;
      }
      g->force_variant = (int32_t)value;
      return DAWN_OK;
    case DAWN_OPT_SELECTOR_MARGIN:
      if (value < 0 || value > 100000) {
        dawn::set_error("selector margin must lie in [0, 100000] thousandths");
        return DAWN_ERR_INVALID_ARG;
      }
      g->sel_margin = (float)value / 1000.0f;
      return DAWN_OK;
    case DAWN_OPT_PULL_SEGMENT:
      if (value < 128 || value > 65536) {
        dawn::set_error("pull segment must lie in [128, 65536]");
        return DAWN_ERR_INVALID_ARG;
      }
      g->pull_seg = (int32_t)value;  // the pull lists and graphs follow on the next call
      return DAWN_OK;
    case DAWN_OPT_BLOCKS_PER_SM:
      if (value < 0 || value > 32) {
        dawn::set_error("CTAs per SM must lie in [0, 32]");
        return DAWN_ERR_INVALID_ARG;
      }
      if (g->blocks_per_sm != (int32_t)value) {
        g->blocks_per_sm = (int32_t)value;
        dawn::drop_graphs(g);  // grid sizes are part of the captured graphs
      }
      return DAWN_OK;
    case DAWN_OPT_AUTO_LEARNED:
      if (value != 0 && value != 1) {
        dawn::set_error("auto-learned must be 0 or 1");
        return DAWN_ERR_INVALID_ARG;
      }
      g->auto_learned = value != 0;
      return DAWN_OK;
    case DAWN_OPT_L2_PERSIST:
      if (value != 0 && value != 1) {
        dawn::set_error("L2 persist must be 0 or 1");
        return DAWN_ERR_INVALID_ARG;
      }
      if (g->l2_persist != (value != 0)) {
        g->l2_persist = value != 0;
        dawn::drop_graphs(g);  // the window is an attribute of the captured kernel nodes
      }
      return DAWN_OK;
    case DAWN_OPT_SMALL_LEVELS:
      if (value != 0 && value != 1) {
        dawn::set_error("small levels must be 0 or 1");
        return DAWN_ERR_INVALID_ARG;
      }
      g->small_levels = value != 0;  // read from the control block at every call
      return DAWN_OK;
    default:
      dawn::set_error("unknown option %d", option);
      return DAWN_ERR_INVALID_ARG;
  }
}

dawn_status dawn_autotune(dawn_graph* g, const int32_t* sources, int32_t nsrc, uint32_t flags, dawn_tuning* out) {
  dawn::clear_error();
  if (!g || !out || nsrc < 1) {
    dawn::set_error("autotune needs a graph, at least one source and an output");
    return DAWN_ERR_INVALID_ARG;
  }
  DAWN_CHECK(check_sources(g, sources, nsrc));
  return dawn::autotune(g, sources, nsrc, flags, out);
}

dawn_status dawn_tune_cache_save(const char* path) {
  dawn::clear_error();
  if (!path) {
    dawn::set_error("path is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  return dawn::tune_cache_save(path);
}

dawn_status dawn_tune_cache_load(const char* path) {
  dawn::clear_error();
  if (!path) {
    dawn::set_error("path is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  return dawn::tune_cache_load(path);
}

dawn_status dawn_graph_set_selector(dawn_graph* g, const float* weights, int32_t count) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  if (!weights) {
    g->sel_on = false;
    return DAWN_OK;
  }
  if (count != DAWN_SELECTOR_WEIGHTS) {
    dawn::set_error("selector needs %d weights, got %d", DAWN_SELECTOR_WEIGHTS, count);
    return DAWN_ERR_INVALID_ARG;
  }
  for (int32_t i = 0; i < count; i++)
    if (!std::isfinite(weights[i])) {
      dawn::set_error("selector weight %d is not finite", i);
      return DAWN_ERR_INVALID_ARG;
    }
  g->sel_user.assign(weights, weights + count);
  g->sel_on = true;
  if (g->sel_slot_state == 1) g->sel_slot_state = 0;  // reload on the next call
  return DAWN_OK;
}

dawn_status dawn_graph_get_option(const dawn_graph* g, int32_t option, int64_t* value) {
  dawn::clear_error();
  if (!g || !value) {
    dawn::set_error("graph or value is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  switch (option) {
    case DAWN_OPT_BITSET_WIDTH:
      *value = g->bs_width;
      return DAWN_OK;
    case DAWN_OPT_PUSH_RATIO:
      *value = g->bs_push_ratio;
      return DAWN_OK;
    case DAWN_OPT_FORCE_VARIANT:
      *value = g->force_variant;
      return DAWN_OK;
    case DAWN_OPT_SELECTOR_MARGIN:
      *value = (int64_t)(g->sel_margin * 1000.0f + 0.5f);
      return DAWN_OK;
    case DAWN_OPT_PULL_SEGMENT:
      *value = g->pull_seg;
      return DAWN_OK;
    case DAWN_OPT_BLOCKS_PER_SM:
      *value = g->blocks_per_sm;
      return DAWN_OK;
    case DAWN_OPT_AUTO_LEARNED:
      *value = g->auto_learned ? 1 : 0;
      return DAWN_OK;
    case DAWN_OPT_L2_PERSIST:
      *value = g->l2_persist ? 1 : 0;
      return DAWN_OK;
    case DAWN_OPT_SMALL_LEVELS:
      *value = g->small_levels ? 1 : 0;
      return DAWN_OK;
    default:
      dawn::set_error("unknown option %d", option);
      return DAWN_ERR_INVALID_ARG;
  }
}

dawn_status dawn_trace_enable(dawn_graph* g, int32_t enable) {
  dawn::clear_error();
  if (!g) {
    dawn::set_error("graph is NULL");
    return DAWN_ERR_INVALID_ARG;
  }
  g->trace = enable != 0;
  return DAWN_OK;
}

dawn_status dawn_trace_read(dawn_graph* g, dawn_trace_rec* out, int64_t cap, int64_t* count) {
  dawn::clear_error();
  if (!g || !count || cap < 0 || (cap > 0 && !out)) {
    dawn::set_error("invalid trace_read arguments");
    return DAWN_ERR_INVALID_ARG;
  }
  const int64_t k = (int64_t)g->trace_log.size() < cap ? (int64_t)g->trace_log.size() : cap;
  if (k > 0) std::memcpy(out, g->trace_log.data(), sizeof(dawn_trace_rec) * (size_t)k);
  g->trace_log.erase(g->trace_log.begin(), g->trace_log.begin() + k);
  *count = k;
  return DAWN_OK;
}

}  // extern "C"
