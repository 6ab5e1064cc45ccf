// rbg_mixed.cu -- mixed-precision form (placeholder until the tcgen05 kernel lands).
#include "rbg_mixed.hpp"

namespace rbg {

int mixed_prepare(const Plan&, const rbg_options&, int64_t, MixedJob&, std::string& err)
{
    err = "mixed precision form not built yet";
    return RBG_ERR_UNSUPPORTED;
}
int mixed_upload(MixedJob&, void*, cudaStream_t, std::string&) { return RBG_ERR_UNSUPPORTED; }
int mixed_launch(const MixedJob&, void*, uint64_t, int64_t, int64_t, double*, cudaStream_t, std::string&)
{
    return RBG_ERR_UNSUPPORTED;
}
int mixed_check(const MixedJob&, void*, cudaStream_t, std::string&) { return RBG_ERR_UNSUPPORTED; }
void mixed_release_cache() {}

}  // namespace rbg
