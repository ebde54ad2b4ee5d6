/*
 * f_vigs_slam/ceres_compat.hpp -- the Ceres cost-function interface the
 * reference's RgbdPoseCostFunction derives from.  With Ceres installed this
 * includes it; without it (no Ceres installed) it declares the
 * two classes with Ceres's shape -- CostFunction with the virtual
 * Evaluate(parameters, residuals, jacobians) and the residual / parameter
 * block sizes, SizedCostFunction<num_residuals, block sizes...> -- so the
 * same cost-function source compiles either way.
 */
#ifndef F_VIGS_SLAM_CERES_COMPAT_HPP
#define F_VIGS_SLAM_CERES_COMPAT_HPP

#if defined(__has_include)
#if __has_include(<ceres/ceres.h>)
#include <ceres/ceres.h>
#define F_VIGS_SLAM_HAVE_CERES 1
#endif
#endif

#ifndef F_VIGS_SLAM_HAVE_CERES
#include <cstdint>
#include <vector>

namespace ceres {

class CostFunction {
public:
    virtual ~CostFunction() = default;
    virtual bool Evaluate(double const* const* parameters, double* residuals, double** jacobians) const = 0;
    const std::vector<int32_t>& parameter_block_sizes() const { return parameter_block_sizes_; }
    int num_residuals() const { return num_residuals_; }

protected:
    std::vector<int32_t>* mutable_parameter_block_sizes() { return &parameter_block_sizes_; }
    void set_num_residuals(int n) { num_residuals_ = n; }

private:
    std::vector<int32_t> parameter_block_sizes_;
    int num_residuals_ = 0;
};

template <int kNumResiduals, int... Ns>
class SizedCostFunction : public CostFunction {
public:
    SizedCostFunction() {
        set_num_residuals(kNumResiduals);
        *mutable_parameter_block_sizes() = std::vector<int32_t>{Ns...};
    }
};

}  // namespace ceres
#endif

#endif
