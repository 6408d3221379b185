// Mixed-precision (tcgen05 tensor-core) form of the Lloyd step.
#include "km_fit.cuh"

namespace kmc {

template <typename T, typename I>
int make_mixed_fit(const FitParams<T, I> &, int, std::unique_ptr<FitBase> *) {
    set_error("the mixed tensor-core form is not available in this build");
    return KMC_ERR_UNSUPPORTED;
}

template int make_mixed_fit<float, int32_t>(const FitParams<float, int32_t> &, int,
                                            std::unique_ptr<FitBase> *);
template int make_mixed_fit<float, int64_t>(const FitParams<float, int64_t> &, int,
                                            std::unique_ptr<FitBase> *);
template int make_mixed_fit<double, int32_t>(const FitParams<double, int32_t> &, int,
                                             std::unique_ptr<FitBase> *);
template int make_mixed_fit<double, int64_t>(const FitParams<double, int64_t> &, int,
                                             std::unique_ptr<FitBase> *);

}  // namespace kmc
