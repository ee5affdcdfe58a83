// A libprofit-style program written against include/profit_cuda.hpp: the
// same calls a user of profit::Model makes (add_profile, parameter,
// set_psf, set_cuda_env, evaluate, create_convolver). It re-runs the
// reference's known-answer tests (tests/test_psf.h:38-50,
// tests/test_sky.h:37-61) and writes a 100x100 sersic model convolved by a
// 15x15 PSF (read from argv[1]) to argv[2] for the caller to compare.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "profit_cuda.hpp"

using namespace profit_cuda;

static int fail(const char *what)
{
	std::cerr << "FAILED: " << what << std::endl;
	return 1;
}

int main(int argc, char **argv)
{
	if (argc != 3) return fail("usage: model_example psf15.bin out.bin");
	auto env = get_cuda_environment(0, true);

	{  // PSF profile known answer: 0.25 in a 2x2 block
		Model m(10, 10);
		m.set_cuda_env(env);
		m.set_psf(Image({1, 1, 1, 1}, 2, 2));
		auto p = m.add_profile("psf");
		p->parameter("xcen", 2.);
		p->parameter("ycen", 2.);
		p->parameter("mag", 0.);
		Image img = m.evaluate();
		for (unsigned int y = 0; y < 10; y++)
			for (unsigned int x = 0; x < 10; x++) {
				const double want = (x >= 1 && x <= 2 && y >= 1 && y <= 2) ? 0.25 : 0.0;
				if (std::fabs(img[x + 10 * y] - want) > 1e-12) return fail("psf known answer");
			}
	}
	{  // sky known answer
		Model m(2, 2);
		m.set_cuda_env(env);
		m.add_profile("sky")->parameter("bg", 1.);
		Image img = m.evaluate();
		for (size_t i = 0; i < img.size(); i++)
			if (img[i] != 1.0) return fail("sky known answer");
	}
	{  // error categories
		Model m(10, 10);
		auto p = m.add_profile("sersic");
		bool thrown = false;
		try {
			p->parameter("fwhm", 1.0);
		}
		catch (const invalid_parameter &) {
			thrown = true;
		}
		if (!thrown) return fail("unknown double parameter must throw invalid_parameter");
		thrown = false;
		try {
			p->parameter("fwhm=1");
		}
		catch (const unknown_parameter &) {
			thrown = true;
		}
		if (!thrown) return fail("unknown spec parameter must throw unknown_parameter");
		p->parameter("axrat", 0.0);
		m.set_cuda_env(env);
		thrown = false;
		try {
			m.evaluate();
		}
		catch (const invalid_parameter &e) {
			thrown = std::string(e.what()).find("axrat") != std::string::npos;
		}
		if (!thrown) return fail("axrat <= 0 must throw invalid_parameter");
	}

	std::vector<double> psf(225);
	std::ifstream in(argv[1], std::ios::binary);
	in.read(reinterpret_cast<char *>(psf.data()), psf.size() * sizeof(double));
	if (!in) return fail("reading the psf");
	Model m(100, 100);
	m.set_cuda_env(env);
	m.set_psf(Image(psf, 15, 15));
	auto s = m.add_profile("sersic");
	s->parameter("xcen", 50.3);
	s->parameter("ycen", 50.7);
	s->parameter("mag", 15.);
	s->parameter("re", 8.);
	s->parameter("nser=4");
	s->parameter("ang", 30.);
	s->parameter("axrat", 0.6);
	s->parameter("convolve", true);
	Image img = m.evaluate();
	std::ofstream out(argv[2], std::ios::binary);
	out.write(reinterpret_cast<const char *>(img.data()), img.size() * sizeof(double));

	auto conv = create_convolver("cuda", env);
	Image src(std::vector<double>(64 * 64, 1.0), 64, 64);
	Image k(std::vector<double>(9, 1.0 / 9), 3, 3);
	Image c = conv->convolve(src, k);
	if (std::fabs(c[32 + 64 * 32] - 1.0) > 1e-14 || std::fabs(c[0] - 4.0 / 9) > 1e-14) return fail("convolver");
	std::cout << "ok" << std::endl;
	return 0;
}
