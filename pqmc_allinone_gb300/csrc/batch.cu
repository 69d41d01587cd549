// batch.cu -- many independent chains in one device context
// (replica parallelism of src/Main_PQMC.f90:373-443 without MPI).
#include <vector>
#include "chain.cuh"

struct pqmc_batch {
  std::vector<pqmc_chain*> chains;
  int precision = PQMC_PREC_FP64;
};

using namespace pqmc;

extern "C" int pqmc_create(const pqmc_model* model, pqmc_chain** out);
extern "C" int pqmc_destroy(pqmc_chain* c);
extern "C" int pqmc_sweep(pqmc_chain* c, int first_loop, int n_sweeps, int warmup, int meas_interval,
                          int meas_number, double* records, int n_records_cap, int* n_records);

extern "C" {

int pqmc_batch_create(const pqmc_model* const* models, int n_chains, int precision, pqmc_batch** out) {
  if (!models || !out || n_chains < 1) { set_error("batch_create: bad arguments"); return PQMC_ERR_ARG; }
  if (precision != PQMC_PREC_FP64 && precision != PQMC_PREC_MIXED) {
    set_error("batch_create: unknown precision %d", precision);
    return PQMC_ERR_ARG;
  }
  pqmc_batch* b = new pqmc_batch();
  b->precision = precision;
  for (int i = 0; i < n_chains; ++i) {
    pqmc_chain* c = nullptr;
    int st = pqmc_create(models[i], &c);
    if (st != PQMC_OK) {
      for (auto* x : b->chains) pqmc_destroy(x);
      delete b;
      return st;
    }
    b->chains.push_back(c);
  }
  *out = b;
  return PQMC_OK;
}

int pqmc_batch_destroy(pqmc_batch* b) {
  if (!b) return PQMC_OK;
  for (auto* c : b->chains) pqmc_destroy(c);
  delete b;
  return PQMC_OK;
}

int pqmc_batch_chain(pqmc_batch* b, int i, pqmc_chain** chain) {
  if (!b || !chain || i < 0 || i >= (int)b->chains.size()) { set_error("batch_chain: bad index"); return PQMC_ERR_ARG; }
  *chain = b->chains[i];
  return PQMC_OK;
}

int pqmc_batch_sweep(pqmc_batch* b, int loop) {
  if (!b) { set_error("null batch"); return PQMC_ERR_ARG; }
  for (auto* c : b->chains) PQMC_TRY(pqmc_sweep(c, loop, 1, 1 << 30, 1, 0, nullptr, 0, nullptr));
  return PQMC_OK;
}

}  // extern "C"
