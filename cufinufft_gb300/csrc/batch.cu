// batch.cu -- the batch C ABI: building the descriptor tables, capturing the
// batch sequence into a CUDA graph and replaying it (kernels in batch.cuh,
// instantiated per precision in batch_f.cu / batch_d.cu).
#include <cmath>

#include "batch.cuh"

namespace cfg {

// Fork: every side stream waits for the work queued so far on b->stream.
template <typename T>
static int fork_sides(Batch<T>* b) {
  CFG_CUDA(cudaEventRecord(b->fork_ev, b->stream));
  for (int k = 0; k < Batch<T>::kSide; ++k) CFG_CUDA(cudaStreamWaitEvent(b->side[k], b->fork_ev, 0));
  return 0;
}
// Join: b->stream waits for everything queued on the side streams.
template <typename T>
static int join_sides(Batch<T>* b) {
  for (int k = 0; k < Batch<T>::kSide; ++k) {
    CFG_CUDA(cudaEventRecord(b->join_ev[k], b->side[k]));
    CFG_CUDA(cudaStreamWaitEvent(b->stream, b->join_ev[k], 0));
  }
  return 0;
}

// The per-plan FFTs, spread over b->stream and the side streams.
template <typename T>
static int batch_ffts(Batch<T>* b) {
  const int n = (int)b->plans.size();
  int e = fork_sides(b);
  if (e) return e;
  for (int i = 0; i < n; ++i) {
    const int br = i % (Batch<T>::kSide + 1);
    cudaStream_t st = br == 0 ? b->stream : b->side[br - 1];
    CFG_CUFFT(cufftSetStream(b->fft[i], st));
    CFG_CUFFT(fft_exec(b->fft[i], b->fw[i], b->plans[i]->iflag));
  }
  return join_sides(b);
}

// Records the whole batch sequence on b->stream (capture or direct); the
// method-1 and method-2 spread/interp kernels run on parallel branches, and
// the FFTs on kSide + 1 branches.
template <typename T>
static int batch_record(Batch<T>* b) {
  const int n = (int)b->plans.size();
  CFG_CUDA(cudaMemcpyAsync(b->d_desc, b->h_desc, sizeof(BatchDesc<T>) * n, cudaMemcpyHostToDevice,
                           b->stream));
  const int rgrid = (int)std::min<long long>(std::max<long long>(b->nrows, 1), 152LL * 16);
  int e = 0;
  if (b->type == 1) {
    for (int i = 0; i < n; ++i) {
      const Plan<T>* p = b->plans[i];
      CFG_CUDA(cudaMemsetAsync(b->fw[i], 0, sizeof(cplx_t<T>) * (size_t)grid_cells(p) * p->ntransf,
                               b->stream));
    }
    if (b->ntasks > 0 || b->nblocks > 0) {
      if ((e = fork_sides(b))) return e;
      CFG_CUDA(batch_spreadinterp(b));
      if ((e = join_sides(b))) return e;
    }
    if ((e = batch_ffts(b))) return e;
    k_batch_deconvolve<T><<<rgrid, 256, 0, b->stream>>>(b->d_desc, n, b->nrows, b->dim);
    CFG_CUDA(cudaGetLastError());
  } else {
    k_batch_amplify<T><<<rgrid, 256, 0, b->stream>>>(b->d_desc, n, b->nrows, b->dim);
    CFG_CUDA(cudaGetLastError());
    if ((e = batch_ffts(b))) return e;
    if (b->ntasks > 0 || b->nblocks > 0) {
      if ((e = fork_sides(b))) return e;
      CFG_CUDA(batch_spreadinterp(b));
      if ((e = join_sides(b))) return e;
    }
  }
  return 0;
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
    b->plans.push_back(p);
  }
  CFG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  CFG_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
  CFG_CUDA(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
  for (int k = 0; k < Batch<T>::kSide; ++k) {
    CFG_CUDA(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
    CFG_CUDA(cudaEventCreateWithFlags(&b->join_ev[k], cudaEventDisableTiming));
  }
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
  if (b->gexec == nullptr) {
    cudaStreamCaptureStatus st;
    bool captured = false;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int e = batch_record(b);
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
      int e = batch_record(b);  // direct launches
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
