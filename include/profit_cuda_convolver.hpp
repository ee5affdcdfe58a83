/*
 * The reference-side binding of the CUDA convolver: a profit::Convolver
 * (include/profit/convolve.h:64-130 of libprofit) whose convolve_impl runs
 * pf_convolve_crop, for the unmodified libprofit's Model::set_convolver
 * (include/profit/model.h:253-255):
 *
 *     #include <profit/profit.h>
 *     #include "profit_cuda_convolver.hpp"
 *     model.set_convolver(std::make_shared<profit::CUDAConvolver>());
 *
 * Unlike include/profit_cuda.hpp (this library's own mirror of the
 * reference's API), this header is compiled against libprofit's headers and
 * linked with libprofit and libpfcuda. Errors of the C ABI become the
 * reference's exceptions (include/profit/exceptions.h:41-104):
 * PF_ERR_INVALID_PARAMETER -> profit::invalid_parameter,
 * PF_ERR_UNKNOWN_PARAMETER -> profit::unknown_parameter, anything else ->
 * profit::cuda_error (a profit::exception, as opencl_error is for OpenCL).
 */
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <profit/convolve.h>
#include <profit/exceptions.h>
#include <profit/image.h>

#include "pf_cuda.h"

namespace profit {

/* A failure of the CUDA backend (device, driver, resources). */
class cuda_error : public exception {
public:
	explicit cuda_error(const std::string &what) : exception(what) {}
};

/* Throws the reference's exception for a non-OK status of the C ABI. */
inline void cuda_check(pf_status status)
{
	if (status == PF_OK) return;
	const std::string msg = pf_last_error();
	if (status == PF_ERR_UNKNOWN_PARAMETER) throw unknown_parameter(msg);
	if (status == PF_ERR_INVALID_PARAMETER) throw invalid_parameter(msg);
	throw cuda_error(msg);
}

/*
 * ConvolverType::CUDA: the direct convolution of pf_convolve_crop on `device`
 * (double precision, the reference's arithmetic order per output pixel).
 * Like BRUTE it adds no padding: crop = false returns the image at offset
 * (0, 0). Images smaller than the kernel are extended by Convolver::convolve
 * before convolve_impl sees them, as for every reference convolver.
 */
class CUDAConvolver : public Convolver {
public:
	explicit CUDAConvolver(int device = 0)
	{
		pf_env *env = nullptr;
		cuda_check(pf_env_create(device, PF_ENV_DOUBLE, &env));
		m_env.reset(env, pf_env_destroy);
	}

protected:
	Image convolve_impl(const Image &src, const Image &krn, const Mask &mask, bool crop, Point &offset_out) override
	{
		const Dimensions sd = src.getDimensions(), kd = krn.getDimensions();
		Image out(sd);
		std::vector<uint8_t> m;
		if (mask) {
			m.resize(mask.size());
			for (unsigned int i = 0; i < mask.size(); i++) m[i] = mask[i] ? 1 : 0;
		}
		uint32_t ox = 0, oy = 0;
		cuda_check(pf_convolve_crop(m_env.get(), src.data(), sd.x, sd.y, krn.data(), kd.x, kd.y,
		                            m.empty() ? nullptr : m.data(), crop ? 1 : 0, out.data(), &ox, &oy));
		if (!crop && &offset_out != &NO_OFFSET) offset_out = Point(ox, oy);
		return out;
	}

private:
	std::shared_ptr<pf_env> m_env;
};

}  // namespace profit
