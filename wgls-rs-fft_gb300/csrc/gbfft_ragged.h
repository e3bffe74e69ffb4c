// Host-side interface of the ragged persistent kernel (fft_ragged.cu).
#pragma once
#include <string>

#include "gbfft_internal.h"

namespace gbfft {

struct RaggedPlanImpl;

// precision: GBFFT_PREC_*; the split forms run the two-pass transforms
// (N = 2^14 .. 2^18) on the tensor cores, the single-pass ones in FP32.
int ragged_plan_build(RaggedPlanImpl *&out, int device, const gbfft_ragged_desc *descs, uint32_t count,
                      int precision, std::string &why);
int ragged_plan_execute(RaggedPlanImpl &p, const void *in, void *out, cudaStream_t stream, bool use_graph,
                        std::string &why);
int ragged_plan_wait(RaggedPlanImpl &p, cudaStream_t stream, std::string &why);
int ragged_plan_set(RaggedPlanImpl &p, int option, uint64_t value, std::string &why);
void ragged_plan_free(RaggedPlanImpl *p);
uint64_t ragged_plan_samples(const RaggedPlanImpl &p);
uint64_t ragged_plan_extent(const RaggedPlanImpl &p);
uint32_t ragged_plan_items(const RaggedPlanImpl &p);
uint64_t ragged_plan_launches(const RaggedPlanImpl &p);

}  // namespace gbfft
