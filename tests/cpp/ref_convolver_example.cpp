// The reference library itself (profit::Model, unmodified) with the CUDA
// convolver of include/profit_cuda_convolver.hpp set through
// Model::set_convolver.
//
//   ref_convolver_example errors   without a GPU: the C ABI's failures reach
//                                  the caller as the reference's exceptions
//   ref_convolver_example render   with a GPU: a sersic model convolved by the
//                                  CUDA convolver equals the same model
//                                  convolved by the reference's BRUTE
//                                  convolver to 1e-12 relative
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>

#include <profit/profit.h>

#include "profit_cuda_convolver.hpp"

static profit::Model sersic_model()
{
	profit::Model model(60, 50);
	auto p = model.add_profile("sersic");
	p->parameter("xcen", 30.3);
	p->parameter("ycen", 24.6);
	p->parameter("mag", 15.0);
	p->parameter("re", 6.0);
	p->parameter("nser", 2.5);
	p->parameter("ang", 30.0);
	p->parameter("axrat", 0.6);
	p->parameter("convolve", true);
	profit::Image psf(9, 9);
	for (unsigned int j = 0; j < 9; j++)
		for (unsigned int i = 0; i < 9; i++) psf[i + j * 9] = std::exp(-((i - 4.) * (i - 4.) + (j - 4.) * (j - 4.)) / 4.);
	model.set_psf(psf);
	return model;
}

int main(int argc, char **argv)
{
	const char *mode = argc > 1 ? argv[1] : "errors";
	if (std::strcmp(mode, "errors") == 0) {
		// an invalid argument of the C ABI: profit::invalid_parameter
		try {
			profit::cuda_check(pf_convolve_crop(nullptr, nullptr, 1, 1, nullptr, 1, 1, nullptr, 1, nullptr, nullptr,
			                                    nullptr));
			std::printf("no exception\n");
			return 1;
		}
		catch (profit::invalid_parameter &e) {
			std::printf("invalid_parameter: %s\n", e.what());
		}
		// no device: a profit::exception (cuda_error), not a crash
		try {
			auto conv = std::make_shared<profit::CUDAConvolver>(0);
			std::printf("device present\n");
		}
		catch (profit::cuda_error &e) {
			std::printf("cuda_error: %s\n", e.what());
		}
		catch (profit::invalid_parameter &e) {
			std::printf("cuda_error expected, got invalid_parameter: %s\n", e.what());
			return 1;
		}
		std::printf("errors ok\n");
		return 0;
	}
	auto model = sersic_model();
	model.set_convolver(profit::create_convolver(profit::ConvolverType::BRUTE));
	const profit::Image want = model.evaluate();
	model.set_convolver(std::make_shared<profit::CUDAConvolver>(0));
	const profit::Image got = model.evaluate();
	double worst = 0;
	for (unsigned int i = 0; i < want.size(); i++) {
		if (want[i] != 0) worst = std::fmax(worst, std::fabs(got[i] - want[i]) / std::fabs(want[i]));
		else if (got[i] != 0) worst = 1;
	}
	std::printf("max rel %.3g\n", worst);
	if (worst > 1e-12) return 1;
	std::printf("render ok\n");
	return 0;
}
