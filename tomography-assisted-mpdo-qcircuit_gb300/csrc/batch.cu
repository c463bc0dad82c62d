// Batched evolution of independent circuits.
//
// One circuit's truncation sweeps are sequential along the chain and launch
// small factorisations (one to a few dozen CTAs each), so a single circuit
// keeps only a fraction of the 152 SMs busy.  Independent circuits overlap:
// the batch runner owns W worker threads, each with its own engine (its own
// non-blocking stream and stream-ordered memory pool) on one device, and
// hands whole circuits to the workers, longest first.  Every worker drives
// the same code path as a single circuit (the public entry points below), so
// a circuit's result does not depend on which worker ran it or on what ran
// beside it.
//
// Host threads never share an engine; the only shared state is the circuit
// counter and the per-circuit status/message slots, each written by one
// worker.
#include "kernels.cuh"
#include "mpdo_gb300.h"

#include <algorithm>
#include <atomic>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

struct mpdo_batch_s {
  int device = 0;
  std::vector<mpdo_engine_t> engines;
  std::vector<std::string> errors;   // message of the last failed circuit per index
};

namespace {

struct Failure {
  mpdo_status st;
};

void ok(mpdo_status s) {
  if (s != MPDO_OK) throw Failure{s};
}

// Relative cost used to order the queue (longest first): per truncate, the
// factorisations of every bond, each of a matrix about 2 kappa chi wide
// (cubic in that width), plus the gate work between truncates.
double cost(const mpdo_program &p) {
  const double chi = p.chi > 0 ? p.chi : 64.0, kap = p.kappa > 0 ? p.kappa : 4.0;
  double ntrunc = 0;
  for (int k = 0; k < p.nops; ++k) ntrunc += p.op_kind[k] == MPDO_OP_TRUNCATE;
  const double w = 2.0 * kap * chi;
  return (ntrunc + 1.0) * p.n * w * w * w + (double)p.nops * w * w;
}

mpdo_status run_one(mpdo_engine_t eng, const mpdo_program &p, mpdo_chain_t *keep) {
  mpdo_chain_t ch = nullptr;
  mpdo_status st = MPDO_OK;
  try {
    ok(mpdo_chain_create(eng, p.n, p.dtype, p.vectors, p.connected, &ch));
    int ntrunc = 0;
    for (int k = 0; k < p.nops; ++k) {
      const double *kr = p.kraus + (p.op_offset ? p.op_offset[k] : 0);
      switch (p.op_kind[k]) {
        case MPDO_OP_1Q: ok(mpdo_apply_1q(ch, p.op_site[k], kr, p.op_k[k])); break;
        case MPDO_OP_2Q: ok(mpdo_apply_2q(ch, p.op_site[k], kr, p.op_k[k], p.abs_cutoff)); break;
        case MPDO_OP_TRUNCATE:
          ok(mpdo_truncate(ch, p.chi, p.kappa, p.max_err, p.noisy,
                           p.discarded ? p.discarded + (size_t)ntrunc * (p.n - 1) : nullptr));
          ++ntrunc;
          break;
        case MPDO_OP_KAPPA: ok(mpdo_kappa_truncate(ch, p.kappa, p.max_err)); break;
        default:
          mpdo::set_last_error("mpdo_batch_run: unknown op kind " + std::to_string(p.op_kind[k]));
          throw Failure{MPDO_ERR_INVALID};
      }
    }
    if (p.z || p.zz) {
      // <Z_i> then <Z_i Z_{i+1}> in one pass over the chain
      const int nz = p.z ? p.n : 0, nzz = p.zz ? p.n - 1 : 0;
      std::vector<int8_t> terms((size_t)(nz + nzz) * p.n, 0);
      for (int i = 0; i < nz; ++i) terms[(size_t)i * p.n + i] = 3;
      for (int i = 0; i < nzz; ++i) {
        terms[(size_t)(nz + i) * p.n + i] = 3;
        terms[(size_t)(nz + i) * p.n + i + 1] = 3;
      }
      std::vector<double> out(nz + nzz);
      if (nz + nzz > 0) ok(mpdo_expect_pauli_batch(ch, terms.data(), nz + nzz, out.data()));
      if (p.z) std::copy(out.begin(), out.begin() + nz, p.z);
      if (p.zz) std::copy(out.begin() + nz, out.end(), p.zz);
    }
    ok(mpdo_engine_sync(eng));
  } catch (const Failure &f) {
    st = f.st;
  } catch (...) {
    mpdo::set_last_error("mpdo_batch_run: unexpected exception");
    st = MPDO_ERR_INVALID;
  }
  if (st == MPDO_OK && keep) {
    *keep = ch;
  } else if (ch) {
    mpdo_chain_destroy(ch);
  }
  return st;
}

}  // namespace

extern "C" {

mpdo_status mpdo_batch_create(int device, int workers, mpdo_batch_t *out) {
  if (!out || workers < 1 || workers > 256) {
    mpdo::set_last_error("mpdo_batch_create: out must be non-NULL and 1 <= workers <= 256");
    return MPDO_ERR_INVALID;
  }
  auto b = std::make_unique<mpdo_batch_s>();
  b->device = device;
  for (int w = 0; w < workers; ++w) {
    mpdo_engine_t e = nullptr;
    mpdo_status st = mpdo_engine_create(device, &e);
    if (st != MPDO_OK) {
      for (auto x : b->engines) mpdo_engine_destroy(x);
      return st;
    }
    b->engines.push_back(e);
  }
  *out = b.release();
  return MPDO_OK;
}

mpdo_status mpdo_batch_destroy(mpdo_batch_t b) {
  if (!b) return MPDO_OK;
  mpdo_status first = MPDO_OK;
  for (auto e : b->engines) {
    mpdo_status st = mpdo_engine_destroy(e);
    if (first == MPDO_OK) first = st;
  }
  delete b;
  return first;
}

mpdo_status mpdo_batch_set_option(mpdo_batch_t b, const char *name, double value) {
  if (!b) {
    mpdo::set_last_error("mpdo_batch_set_option: batch is NULL");
    return MPDO_ERR_INVALID;
  }
  for (auto e : b->engines) {
    mpdo_status st = mpdo_engine_set_option(e, name, value);
    if (st != MPDO_OK) return st;
  }
  return MPDO_OK;
}

mpdo_status mpdo_batch_num_workers(mpdo_batch_t b, int *workers) {
  if (!b || !workers) {
    mpdo::set_last_error("mpdo_batch_num_workers: NULL argument");
    return MPDO_ERR_INVALID;
  }
  *workers = (int)b->engines.size();
  return MPDO_OK;
}

mpdo_status mpdo_batch_engine(mpdo_batch_t b, int worker, mpdo_engine_t *out) {
  if (!b || !out || worker < 0 || worker >= (int)b->engines.size()) {
    mpdo::set_last_error("mpdo_batch_engine: bad batch, worker index or out pointer");
    return MPDO_ERR_INVALID;
  }
  *out = b->engines[worker];
  return MPDO_OK;
}

mpdo_status mpdo_batch_run(mpdo_batch_t b, int ncirc, const mpdo_program *progs, mpdo_chain_t *chains_out,
                           int *worker_out, int *status_out) {
  if (!b || ncirc < 0 || (ncirc > 0 && !progs)) {
    mpdo::set_last_error("mpdo_batch_run: bad batch or program array");
    return MPDO_ERR_INVALID;
  }
  for (int i = 0; i < ncirc; ++i) {
    const mpdo_program &p = progs[i];
    if (p.n < 1 || (p.dtype != MPDO_C64 && p.dtype != MPDO_C128) || !p.vectors || p.nops < 0 ||
        (p.nops > 0 && (!p.op_kind || !p.op_site || !p.op_k))) {
      mpdo::set_last_error("mpdo_batch_run: program " + std::to_string(i) + " is malformed");
      return MPDO_ERR_INVALID;
    }
  }
  std::vector<int> order(ncirc);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost(progs[a]) > cost(progs[c]); });
  std::vector<mpdo_status> st(ncirc, MPDO_OK);
  b->errors.assign(ncirc, std::string());
  if (chains_out)
    for (int i = 0; i < ncirc; ++i) chains_out[i] = nullptr;
  std::atomic<int> next{0};
  const int W = std::min<int>((int)b->engines.size(), std::max(ncirc, 1));
  auto worker = [&](int w) {
    cudaSetDevice(b->device);
    for (;;) {
      const int j = next.fetch_add(1);
      if (j >= ncirc) break;
      const int i = order[j];
      st[i] = run_one(b->engines[w], progs[i], chains_out ? &chains_out[i] : nullptr);
      if (st[i] != MPDO_OK) b->errors[i] = mpdo_last_error();
      if (worker_out) worker_out[i] = w;
    }
  };
  std::vector<std::thread> threads;
  for (int w = 1; w < W; ++w) threads.emplace_back(worker, w);
  // worker 0 runs on the calling thread and selects the batch's device: the
  // caller's current device is restored afterwards
  int caller_dev = -1;
  if (cudaGetDevice(&caller_dev) != cudaSuccess) { cudaGetLastError(); caller_dev = -1; }
  worker(0);
  for (auto &t : threads) t.join();
  if (caller_dev >= 0) cudaSetDevice(caller_dev);
  mpdo_status first = MPDO_OK;
  for (int i = 0; i < ncirc; ++i) {
    if (status_out) status_out[i] = st[i];
    if (first == MPDO_OK && st[i] != MPDO_OK) {
      first = st[i];
      mpdo::set_last_error("circuit " + std::to_string(i) + ": " + b->errors[i]);
    }
  }
  return first;
}

const char *mpdo_batch_error(mpdo_batch_t b, int circuit) {
  if (!b || circuit < 0 || circuit >= (int)b->errors.size()) return "";
  return b->errors[circuit].c_str();
}

}  // extern "C"
