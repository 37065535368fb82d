// Internal interface of the conventional (stored-integral) build (store.cu), used by the C ABI in
// context.cu.
#pragma once
#include <string>

#include "../../include/unomol_gb300.h"
#include "ctx_view.h"

namespace ugb {

struct IntStore;

// A store from the context's own integrals (record pass on the device), or from a file of 24-byte
// records.  max_gib bounds the device memory the construction holds at once.  Status codes of the C ABI;
// err gets the message.
int store_from_integrals(const CtxView& v, int kind, double max_gib, IntStore** out, std::string& err);
int store_from_file(const CtxView& v, const char* path, int kind, double max_gib, IntStore** out, std::string& err);
// The canonical records of the context's basis, written to `path` as raw 24-byte records.
int write_records(const CtxView& v, const char* path, long long* count, std::string& err);
// G += the stored map applied to P (packed device arrays; dPb / dGb null for RHF).  A UHF build needs a
// UNOMOL_STORE_UHF store.  *launches counts the kernels.
cudaError_t store_fock(const IntStore* st, const double* dPa, const double* dPb, double* dGa, double* dGb, cudaStream_t s,
                       int* launches);
int store_kind(const IntStore* st);
double store_max_gib(const IntStore* st);
void store_info(const IntStore* st, UnomolStoreInfo* out);
void store_free(IntStore* st);

}  // namespace ugb
