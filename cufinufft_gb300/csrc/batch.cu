// batch.cu -- the batch C ABI: building the descriptor tables, capturing the
// batch sequence into a CUDA graph and replaying it (kernels in batch.cuh,
// instantiated per precision in batch_f.cu / batch_d.cu).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "batch.cuh"

namespace cfg {

// An event of the recorded sequence (a fresh one per record or wait pair,
// so every dependency of the captured graph is explicit).
template <typename T>
static cudaError_t next_event(Batch<T>* b, cudaEvent_t* ev) {
  if (b->evnext == b->evpool.size()) {
    cudaEvent_t e;
    const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (r != cudaSuccess) return r;
    b->evpool.push_back(e);
  }
  *ev = b->evpool[b->evnext++];
  return cudaSuccess;
}

// `to` waits for everything queued so far on `from`.
template <typename T>
static cudaError_t follow(Batch<T>* b, cudaStream_t from, cudaStream_t to) {
  cudaEvent_t e;
  cudaError_t r = next_event(b, &e);
  if (r == cudaSuccess) r = cudaEventRecord(e, from);
  if (r == cudaSuccess) r = cudaStreamWaitEvent(to, e, 0);
  return r;
}

// Spread/interp kernels of one group: side[0] and side[1] fork from and join
// back into b->stream.
template <typename T>
static int group_spreadinterp(Batch<T>* b, const BatchGroup& g) {
  if (g.t1 <= g.t0 && g.b1 <= g.b0) return 0;
  CFG_CUDA(follow(b, b->stream, b->side[0]));
  CFG_CUDA(follow(b, b->stream, b->side[1]));
  CFG_CUDA(batch_spreadinterp(b, g));
  CFG_CUDA(follow(b, b->side[0], b->stream));
  CFG_CUDA(follow(b, b->side[1], b->stream));
  return 0;
}

// FFT stream of plan i: the kFftSide FFT streams in turn.
template <typename T>
static cudaStream_t fft_stream(Batch<T>* b, int i) {
  return b->side[2 + i % Batch<T>::kFftSide];
}

// The FFTs of plans [p0, p1), each on its plan's FFT stream after the work
// queued so far on b->stream; returns (in *joined) the stream of plan p0,
// made to wait for all of them.
template <typename T>
static int group_ffts(Batch<T>* b, int p0, int p1, cudaStream_t* joined) {
  const int used = std::min(p1 - p0, Batch<T>::kFftSide);
  for (int i = p0; i < p0 + used; ++i) {
    CFG_CUDA(follow(b, b->stream, fft_stream(b, i)));
    b->fft_used |= 1u << (i % Batch<T>::kFftSide);
  }
  for (int i = p0; i < p1; ++i) {
    CFG_CUFFT(cufftSetStream(b->fft[i], fft_stream(b, i)));
    CFG_CUFFT(fft_exec(b->fft[i], b->fw[i], b->plans[i]->iflag));
  }
  cudaStream_t a = fft_stream(b, p0);
  for (int i = p0 + 1; i < p0 + used; ++i) CFG_CUDA(follow(b, fft_stream(b, i), a));
  *joined = a;
  return 0;
}

static int row_blocks(long long rows) {
  return (int)std::min<long long>(std::max<long long>(rows, 1), 152LL * 16);
}

// Records the whole batch sequence on b->stream (capture or direct).
// Type 1 runs its groups as a pipeline: group g's spread kernels on b->stream
// (and side[0], side[1]); then its FFTs on the FFT streams and its
// deconvolution behind them while group g + 1 is spread.  Type 2 amplifies
// every plan, runs every FFT and interpolates, one stage after the other.
template <typename T>
static int batch_record(Batch<T>* b) {
  const int n = (int)b->plans.size();
  b->evnext = 0;
  b->fft_used = 0;
  CFG_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc, sizeof(BatchDesc<T>) * n, cudaMemcpyHostToDevice,
                           b->stream));
  int e = 0;
  if (b->type == 1) {
    for (int i = 0; i < n; ++i) {
      const Plan<T>* p = b->plans[i];
      CFG_CUDA(cudaMemsetAsync(b->fw[i], 0, sizeof(cplx_t<T>) * (size_t)grid_cells(p) * p->ntransf,
                               b->stream));
    }
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
      const BatchGroup& g = b->groups[gi];
      if ((e = group_spreadinterp(b, g))) return e;
      cudaStream_t a = nullptr;
      if ((e = group_ffts(b, g.p0, g.p1, &a))) return e;
      if (g.r1 > g.r0) {
        k_batch_deconvolve<T><<<row_blocks(g.r1 - g.r0), 256, 0, a>>>(b->d_desc, n, g.r0, g.r1, b->dim);
        CFG_CUDA(cudaGetLastError());
      }
    }
    // join the FFT streams this sequence used (an unused one never joined
    // the capture)
    for (int k = 0; k < Batch<T>::kFftSide; ++k)
      if (b->fft_used & (1u << k)) CFG_CUDA(follow(b, b->side[2 + k], b->stream));
  } else {
    const BatchGroup all = {0, n, 0, b->ntasks, 0, b->nblocks, 0, b->nrows};
    k_batch_amplify<T><<<row_blocks(b->nrows), 256, 0, b->stream>>>(b->d_desc, n, 0, b->nrows, b->dim);
    CFG_CUDA(cudaGetLastError());
    cudaStream_t a = nullptr;
    if ((e = group_ffts(b, 0, n, &a))) return e;
    CFG_CUDA(follow(b, a, b->stream));
    if ((e = group_spreadinterp(b, all))) return e;
  }
  return 0;
}

// The batch as every plan's own execute: plans go, heaviest first, to the
// least-loaded of the kSide branch streams (load = taps + grid cells), each
// running its own tuned spread/interp kernels, cuFFT plans and
// deconvolution there.
template <typename T>
static int batch_record_plans(Batch<T>* b, cplx_t<T>** c, cplx_t<T>** fk) {
  const int n = (int)b->plans.size();
  constexpr int K = Batch<T>::kSide;
  b->evnext = 0;
  std::vector<double> w(n);
  std::vector<int> order(n), branch(n);
  for (int i = 0; i < n; ++i) {
    const Plan<T>* p = b->plans[i];
    w[i] = (double)p->M * p->ntransf * std::pow((double)p->sp.ns, p->dim) +
           8.0 * (double)grid_cells(p) * p->ntransf + 1.0;
    order[i] = i;
  }
  std::sort(order.begin(), order.end(), [&](int x, int y) { return w[x] > w[y]; });
  double load[K] = {};
  for (int i : order) {
    int k = 0;
    for (int q = 1; q < K; ++q)
      if (load[q] < load[k]) k = q;
    branch[i] = k;
    load[k] += w[i];
  }
  for (int k = 0; k < K; ++k)
    if (load[k] > 0) CFG_CUDA(follow(b, b->stream, b->side[k]));
  for (int i : order) {
    Plan<T>* p = b->plans[i];
    cudaStream_t own = p->stream;
    int e = plan_use_stream(p, b->side[branch[i]]);
    if (!e) e = execute_plan(p, c[i], fk[i]);
    const int e2 = plan_use_stream(p, own);
    if (e) return e;
    if (e2) return e2;
  }
  for (int k = 0; k < K; ++k)
    if (load[k] > 0) CFG_CUDA(follow(b, b->side[k], b->stream));
  return 0;
}

// Type-1 groups: consecutive plans cut where the running tap count (M ntr
// ns^d per plan) crosses k / kBatchGroups of the total, so each group's spread
// is about as long and its FFTs overlap the next group's spreading.
constexpr int kBatchGroups = 4;

template <typename T>
static void make_groups(Batch<T>* b) {
  const int n = (int)b->plans.size();
  b->groups.clear();
  auto group_of = [&](int p0, int p1) {
    BatchGroup g;
    g.p0 = p0;
    g.p1 = p1;
    g.t0 = b->h_desc[p0].task0;
    g.b0 = b->h_desc[p0].blk0;
    g.r0 = b->h_desc[p0].row0;
    g.t1 = p1 < n ? b->h_desc[p1].task0 : b->ntasks;
    g.b1 = p1 < n ? b->h_desc[p1].blk0 : b->nblocks;
    g.r1 = p1 < n ? b->h_desc[p1].row0 : b->nrows;
    return g;
  };
  if (b->type != 1) {
    b->groups.push_back(group_of(0, n));
    return;
  }
  std::vector<double> w(n);
  double total = 0;
  for (int i = 0; i < n; ++i) {
    const Plan<T>* p = b->plans[i];
    w[i] = (double)p->M * p->ntransf * std::pow((double)p->sp.ns, p->dim) + 1.0;
    total += w[i];
  }
  const int G = std::min(n, kBatchGroups);
  double acc = 0;
  int p0 = 0;
  for (int i = 0; i < n; ++i) {
    acc += w[i];
    const int k = (int)b->groups.size() + 1;
    if (i + 1 < n && k < G && acc >= total * k / G) {
      b->groups.push_back(group_of(p0, i + 1));
      p0 = i + 1;
    }
  }
  b->groups.push_back(group_of(p0, n));
}

template <typename T>
static int batch_make(Batch<T>* b, int nplans, Plan<T>** plans) {
  if (nplans < 1 || plans == nullptr) return CUFINUFFT_ERR_ARG;
  for (int i = 0; i < nplans; ++i) {
    Plan<T>* p = plans[i];
    if (!p || !p->planned || !p->pts_set) return CUFINUFFT_ERR_GENERIC;
    if (i == 0) {
      b->type = p->type;
      b->dim = p->dim;
      b->ns = p->sp.ns;
      b->device = p->device;
    }
    if (p->type != b->type || p->dim != b->dim || p->sp.ns != b->ns || p->device != b->device)
      return CUFINUFFT_ERR_ARG;  // one type, dimension, kernel width and device per batch
    if (p->opts.gpu_kerevalmeth != 0) return CUFINUFFT_ERR_ARG;
    if (p->spread_only) return CUFINUFFT_ERR_ARG;  // the batch runs whole transforms
    if (p->type == 3) return CUFINUFFT_ERR_ARG;    // types 1 and 2 only
    b->plans.push_back(p);
  }
  CFG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  CFG_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
  for (int k = 0; k < Batch<T>::kSide; ++k)
    CFG_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
  // default: the graph of each plan's own execute; CUFINUFFT_BATCH=tables
  // selects the multi-plan kernels over descriptor tables
  const char* mode = std::getenv("CUFINUFFT_BATCH");
  b->by_plans = !(mode && std::strcmp(mode, "tables") == 0);
  if (b->by_plans) return 0;
  for (Plan<T>* p : b->plans)
    if (p->lo) return CUFINUFFT_ERR_ARG;  // the tables hold FP64 grids; an FP32 chain has none
  CFG_CUDA(cudaMallocHost(&b->h_desc, sizeof(BatchDesc<T>) * nplans));
  CFG_CUDA(cudaMalloc(&b->d_desc, sizeof(BatchDesc<T>) * nplans));
  long long task = 0, row = 0, blk = 0;
  for (int i = 0; i < nplans; ++i) {
    Plan<T>* p = b->plans[i];
    cplx_t<T>* fw = nullptr;
    CFG_CUDA(cudaMalloc(&fw, sizeof(cplx_t<T>) * (size_t)grid_cells(p) * p->ntransf));
    b->fw.push_back(fw);
    cufftHandle h;
    int nn[3], dist = (int)grid_cells(p);
    for (int k = 0; k < p->dim; ++k) nn[k] = p->nf[p->dim - 1 - k];
    CFG_CUFFT(cufftPlanMany(&h, p->dim, nn, nn, 1, dist, nn, 1, dist, fft_type<T>(), p->ntransf));
    b->fft.push_back(h);
    CFG_CUFFT(cufftSetStream(h, b->stream));
    BatchDesc<T>& D = b->h_desc[i];
    std::memset(&D, 0, sizeof(D));
    D.M = p->M;
    D.ntr = p->ntransf;
    for (int k = 0; k < 3; ++k) {
      D.nf[k] = p->nf[k];
      D.N[k] = p->N[k];
      D.i0[k] = p->i0[k];
      D.d[k] = p->d[k];
      D.fac[k] = p->fac[k];
    }
    D.Nf = grid_cells(p);
    D.Nm = (long long)p->N[0] * p->N[1] * p->N[2];
    D.idx = p->idx;
    D.beta = (T)p->sp.beta;
    D.c = (T)p->sp.c;
    D.e_beta = (T)std::exp(p->sp.beta);
    D.bl2e = (T)(p->sp.beta * 1.44269504088896340736);
    D.fw = fw;
    D.task0 = task;
    D.row0 = row;
    D.blk0 = blk;
    D.method = (p->method == 2 && p->nsub > 0) ? 2 : 1;
    if (p->method == 2 && p->nsub == 0 && p->M > 0) D.method = 1;
    // points per warp step: spreading uses ns-wide lane groups,
    // interpolation power-of-two groups (see spreadinterp.cuh)
    const int L = b->type == 1 ? b->ns : (b->ns <= 2 ? 2 : (b->ns <= 4 ? 4 : (b->ns <= 8 ? 8 : 16)));
    const int PPW = 32 / L;
    if (D.method == 1) {
      task += ((long long)p->M + PPW - 1) / PPW;
    } else {
      for (int k = 0; k < 3; ++k) {
        D.bins.bs[k] = p->bs[k];
        D.bins.nb[k] = p->nb[k];
      }
      D.bins.nbins = p->nbins;
      D.bins.count = p->count;
      D.bins.start = p->start;
      D.bins.sub_start = p->sub_start;
      D.bins.sub_to_bin = p->sub_to_bin;
      D.bins.nsub = p->nsub;
      D.bins.maxsub = p->opts.gpu_maxsubprobsize;
      blk += (long long)p->nsub * p->ntransf;
      b->smem = std::max(b->smem, tile_cells(p->dim, p->sp.ns, p->bs) * sizeof(cplx_t<T>));
      if (b->type == 1 && p->cell_order && p->sub_dense) {
        D.sub_dense = p->sub_dense;
        BinTables bt;
        std::memset(&bt, 0, sizeof(bt));
        for (int k = 0; k < 3; ++k) bt.bs[k] = p->bs[k];
        const size_t rb = p->dim == 1 ? run_bytes<T, 1>(p->sp.ns, bt)
                          : (p->dim == 2 ? run_bytes<T, 2>(p->sp.ns, bt) : run_bytes<T, 3>(p->sp.ns, bt));
        b->smem_run = std::max(b->smem_run, rb);
      }
    }
    row += (b->type == 1 ? (long long)p->N[1] * p->N[2] : (long long)p->nf[1] * p->nf[2]) * p->ntransf;
  }
  b->ntasks = task;
  b->nrows = row;
  b->nblocks = blk;
  make_groups(b);
  return 0;
}

template <typename T>
static int batch_execute(Batch<T>* b, cplx_t<T>** c, cplx_t<T>** fk) {
  const int n = (int)b->plans.size();
  if (c == nullptr || fk == nullptr) return CUFINUFFT_ERR_ARG;
  // the previous replay must have copied the descriptor table before it is
  // rewritten
  if (b->launched) CFG_CUDA(cudaEventSynchronize(b->done));
  for (int i = 0; i < n; ++i) {
    if ((b->plans[i]->M > 0 && c[i] == nullptr) || fk[i] == nullptr) return CUFINUFFT_ERR_ARG;
    if (b->by_plans) continue;
    BatchDesc<T>& D = b->h_desc[i];
    if (b->type == 1) {
      D.c_in = c[i];
      D.c_out = nullptr;
    } else {
      D.c_in = nullptr;
      D.c_out = c[i];
    }
    D.fk = fk[i];
  }
  // order after the legacy default stream, as a plan's stream is
  CFG_CUDA(cudaEventRecord(b->done, cudaStreamLegacy));
  CFG_CUDA(cudaStreamWaitEvent(b->stream, b->done, 0));
  if (b->by_plans && b->gexec != nullptr &&
      !(std::equal(b->cap_c.begin(), b->cap_c.end(), c) && std::equal(b->cap_fk.begin(), b->cap_fk.end(), fk))) {
    // other caller arrays: capture again
    cudaGraphExecDestroy(b->gexec);
    cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
  }
  if (b->gexec == nullptr) {
    cudaStreamCaptureStatus st;
    bool captured = false;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int e = b->by_plans ? batch_record_plans(b, c, fk) : batch_record(b);
      if (b->by_plans) {
        b->cap_c.assign(c, c + n);
        b->cap_fk.assign(fk, fk + n);
      }
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
      if (e == 0 && ce == cudaSuccess && g != nullptr &&
          cudaGraphInstantiate(&b->gexec, g, 0) == cudaSuccess) {
        b->graph = g;
        captured = true;
      } else if (g) {
        cudaGraphDestroy(g);
      }
      (void)st;
    }
    cudaGetLastError();
    if (!captured) {
      b->gexec = nullptr;
      int e = b->by_plans ? batch_record_plans(b, c, fk) : batch_record(b);  // direct launches
      if (e) return e;
      CFG_CUDA(cudaEventRecord(b->done, b->stream));
      b->launched = true;
      CFG_CUDA(cudaStreamWaitEvent(cudaStreamLegacy, b->done, 0));
      return 0;
    }
  }
  CFG_CUDA(cudaGraphLaunch(b->gexec, b->stream));
  CFG_CUDA(cudaEventRecord(b->done, b->stream));
  b->launched = true;
  // later work on the legacy default stream sees the results
  CFG_CUDA(cudaStreamWaitEvent(cudaStreamLegacy, b->done, 0));
  return 0;
}

}  // namespace cfg

struct cufinufft_batch_s {
  cfg::Batch<double> b;
};
struct cufinufftf_batch_s {
  cfg::Batch<float> b;
};

template <typename H, typename PH, typename T>
static int batch_make_entry(int nplans, PH** plans, H** out) {
  if (out == nullptr) return CUFINUFFT_ERR_ARG;
  *out = nullptr;
  if (nplans < 1 || plans == nullptr) return CUFINUFFT_ERR_ARG;
  std::vector<cfg::Plan<T>*> ps(nplans);
  for (int i = 0; i < nplans; ++i) {
    if (plans[i] == nullptr) return CUFINUFFT_ERR_ARG;
    ps[i] = &plans[i]->p;
  }
  H* h = new H();
  cfg::DeviceGuard g(ps[0]->device);
  int e = cfg::batch_make<T>(&h->b, nplans, ps.data());
  if (e) {
    cfg::batch_release(&h->b);
    delete h;
    return e;
  }
  *out = h;
  return 0;
}

extern "C" {

int cufinufft_batch_make(int nplans, cufinufft_plan* plans, cufinufft_batch* batch) {
  return batch_make_entry<cufinufft_batch_s, cufinufft_plan_s, double>(nplans, plans, batch);
}
int cufinufftf_batch_make(int nplans, cufinufftf_plan* plans, cufinufftf_batch* batch) {
  return batch_make_entry<cufinufftf_batch_s, cufinufftf_plan_s, float>(nplans, plans, batch);
}

int cufinufft_batch_execute(cufinufft_batch batch, cuDoubleComplex** c, cuDoubleComplex** fk) {
  if (!batch) return CUFINUFFT_ERR_GENERIC;
  cfg::DeviceGuard g(batch->b.device);
  return cfg::batch_execute(&batch->b, reinterpret_cast<double2**>(c), reinterpret_cast<double2**>(fk));
}
int cufinufftf_batch_execute(cufinufftf_batch batch, cuFloatComplex** c, cuFloatComplex** fk) {
  if (!batch) return CUFINUFFT_ERR_GENERIC;
  cfg::DeviceGuard g(batch->b.device);
  return cfg::batch_execute(&batch->b, reinterpret_cast<float2**>(c), reinterpret_cast<float2**>(fk));
}

int cufinufft_batch_destroy(cufinufft_batch batch) {
  if (!batch) return 1;
  {
    cfg::DeviceGuard g(batch->b.device);
    cudaStreamSynchronize(batch->b.stream);
    cfg::batch_release(&batch->b);
  }
  delete batch;
  return 0;
}
int cufinufftf_batch_destroy(cufinufftf_batch batch) {
  if (!batch) return 1;
  {
    cfg::DeviceGuard g(batch->b.device);
    cudaStreamSynchronize(batch->b.stream);
    cfg::batch_release(&batch->b);
  }
  delete batch;
  return 0;
}

}  // extern "C"
