// profit-cli for the CUDA backend: profit-cli's command line
// (src/profit-cli.cpp of libprofit) on this library's C++ interface
// (include/profit_cuda.hpp), for running and timing models from a shell.
//
//   profit-cli -p sersic:xcen=50:ycen=50:re=8:nser=4 -P psf.fits -f out.fits
//   profit-cli -w 1000 -H 1000 -p sersic:... -p sky:bg=1e-3 -T fft -i 100 -s
//
// Options as the reference's, -T selecting this backend's convolutions and -D
// its precision; OpenCL, FFTW and SIMD options do not apply.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include <unistd.h>

#include "profit_cuda.hpp"

namespace profit = profit_cuda;

namespace {

const char *kUsage = R"(%s: generates an image from a model and its profiles on a CUDA device

Usage: %s [options] -p <spec> [-p <spec> ...]

Options:
  -t        Output image as text values on stdout (17 significant digits)
  -f <file> Output image as a FITS file
  -i <n>    Evaluate the model n times and report the time taken
  -s        Show runtime stats (Model::get_stats)
  -T <conv> Convolver: brute (or cuda), fft (or cuda-fft), auto. Defaults to auto
  -u        Return an un-cropped image from the convolver
  -D <0|1>  Double precision (1, the default: the reference's arithmetic) or
            single precision with FP64 where it decides the result (0)
  -d <n>    CUDA device. Defaults to 0
  -w        Width in pixels. Defaults to 100
  -H        Height in pixels. Defaults to 100
  -x        Image width in image coordinates. Defaults to the width in pixels
  -y        Image height in image coordinates. Defaults to the height in pixels
  -S <n>    Finesampling factor. Defaults to 1
  -F        Do *not* return finesampled image (if -S <n>)
  -m        Zero magnitude. Defaults to 0
  -P        PSF (as w:h:val1,val2,..., or a FITS file name)
  -h,-?     Show this help and exit
  -V        Show the program version and exit

Profiles are given as [count,]name[:param1=val1:param2=val2:...], count the
number of copies of the profile. Profiles: sersic, coresersic, moffat, ferrer,
king, brokenexp, sky, psf, null, with the reference's parameter names.
)";

std::vector<std::string> split(const std::string &s, char sep)
{
	std::vector<std::string> out;
	std::string cur;
	std::istringstream in(s);
	while (std::getline(in, cur, sep)) out.push_back(cur);
	return out;
}

void add_profiles(profit::Model &m, const std::string &spec)
{
	if (spec.empty()) throw profit::invalid_parameter("Missing parameter name after -p");
	unsigned int count = 1;
	std::string rest = spec;
	const auto comma = spec.find(',');
	if (comma != std::string::npos) {
		count = (unsigned int)std::stod(spec.substr(0, comma));
		rest = spec.substr(comma + 1);
	}
	const auto parts = split(rest, ':');
	for (unsigned int c = 0; c < count; c++) {
		auto p = m.add_profile(parts[0]);
		for (size_t i = 1; i < parts.size(); i++) {
			try {
				p->parameter(parts[i]);
			}
			catch (const profit::unknown_parameter &e) {
				std::cerr << e.what() << std::endl;
			}
		}
	}
}

profit::Image read_psf(const std::string &arg, profit::PixelScale &scale)
{
	const auto parts = split(arg, ':');
	if (parts.size() >= 3) {  // w:h:v1,v2,...
		const unsigned int w = (unsigned int)std::stoul(parts[0]), h = (unsigned int)std::stoul(parts[1]);
		const auto vals = split(parts[2], ',');
		if (vals.size() != (size_t)w * h) throw profit::invalid_parameter("PSF needs w x h values");
		std::vector<double> v;
		for (const auto &x : vals) v.push_back(std::stod(x));
		return profit::Image(v, w, h);
	}
	return profit::from_fits(arg, scale);
}

void stats_line(const std::string &prefix, const std::string &name, double ms)
{
	std::string label = prefix + name;
	if (label.size() < 50) label += std::string(50 - label.size(), ' ');
	std::cout << label << " : " << std::setw(10) << std::setprecision(3) << std::fixed << ms << " [ms]" << std::endl;
}

}  // namespace

int main(int argc, char **argv)
{
	unsigned int width = 100, height = 100, fs = 1, iterations = 1;
	double xsize = -1, ysize = -1;
	bool text = false, stats = false, uncropped = false, double_precision = true, return_fs = true;
	int device = 0;
	std::string fits_out, convolver = "auto";
	profit::Model m;
	profit::Image psf;
	profit::PixelScale psf_scale{1, 1};
	bool have_psf = false;
	int opt;
	try {
		while ((opt = getopt(argc, argv, "h?Vtf:i:sT:uD:d:w:H:x:y:S:Fm:P:p:")) != -1) {
			switch (opt) {
			case 'h':
			case '?':
				std::printf(kUsage, argv[0], argv[0]);
				return opt == 'h' ? 0 : 1;
			case 'V':
				std::printf("profit-cli (CUDA backend) %s\n", pf_version());
				return 0;
			case 't': text = true; break;
			case 'f': fits_out = optarg; break;
			case 'i': iterations = (unsigned int)std::stoul(optarg); break;
			case 's': stats = true; break;
			case 'T': convolver = optarg; break;
			case 'u': uncropped = true; break;
			case 'D': double_precision = std::atoi(optarg) != 0; break;
			case 'd': device = std::atoi(optarg); break;
			case 'w': width = (unsigned int)std::stoul(optarg); break;
			case 'H': height = (unsigned int)std::stoul(optarg); break;
			case 'x': xsize = std::stod(optarg); break;
			case 'y': ysize = std::stod(optarg); break;
			case 'S': fs = (unsigned int)std::stoul(optarg); break;
			case 'F': return_fs = false; break;
			case 'm': m.set_magzero(std::stod(optarg)); break;
			case 'P':
				psf = read_psf(optarg, psf_scale);
				have_psf = true;
				break;
			case 'p': add_profiles(m, optarg); break;
			default:
				std::printf(kUsage, argv[0], argv[0]);
				return 1;
			}
		}
		if (!m.has_profiles()) {
			std::printf(kUsage, argv[0], argv[0]);
			return 1;
		}
		m.set_dimensions(width, height);
		m.set_image_pixel_scale({xsize > 0 ? xsize / width : 1.0, ysize > 0 ? ysize / height : 1.0});
		m.set_finesampling(fs);
		m.set_return_finesampled(return_fs);
		m.set_crop(!uncropped);
		m.set_convolver(convolver);
		if (have_psf) {
			m.set_psf(psf);
			m.set_psf_pixel_scale(psf_scale);
		}
		auto t0 = std::chrono::steady_clock::now();
		m.set_cuda_env(profit::get_cuda_environment(device, double_precision, stats));
		auto t1 = std::chrono::steady_clock::now();
		std::cout << "CUDA environment (device " << device << ", " << (double_precision ? "double" : "single")
		          << " precision) created in " << std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count()
		          << " [ms]" << std::endl;
		std::pair<unsigned int, unsigned int> offset;
		profit::Image image;
		t0 = std::chrono::steady_clock::now();
		for (unsigned int i = 0; i < iterations; i++) image = m.evaluate(offset);
		t1 = std::chrono::steady_clock::now();
		const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
		std::cout << std::fixed << std::setprecision(3) << "Ran " << iterations << " iterations in " << ms / 1000
		          << " [s] (" << ms / iterations << " [ms] per iteration)" << std::endl;
		if (text) {
			// every value with 17 significant digits (round trips through text)
			std::cout << std::defaultfloat << std::setprecision(17);
			for (unsigned int j = 0; j < image.getHeight(); j++) {
				for (unsigned int i = 0; i < image.getWidth(); i++) std::cout << image[j * image.getWidth() + i] << " ";
				std::cout << std::endl;
			}
		}
		if (!fits_out.empty()) {
			profit::Point p;
			p.x = offset.first;
			p.y = offset.second;
			profit::to_fits(image, p, m.get_image_pixel_scale(), fits_out);
		}
		if (stats) {
			std::cout << std::endl;
			for (const auto &kv : m.get_stats()) {
				const auto *rs = dynamic_cast<const profit::RadialProfileStats *>(kv.second.get());
				std::cout << "Stats for profile " << kv.first << std::endl;
				if (rs) {
					stats_line("", "Setup pass (all profiles)", rs->cuda_times.setup / 1e6);
					stats_line("", "Evaluation pass (all profiles)", rs->cuda_times.evaluation / 1e6);
					stats_line("", "Convolution pass (all profiles)", rs->cuda_times.convolution / 1e6);
					std::cout << "  evaluate_at calls: " << rs->evaluations << std::endl;
					for (const auto &lv : rs->integrations)
						std::cout << "  Level " << lv.first << ": " << lv.second << " integrations" << std::endl;
				}
				stats_line("", "Total", kv.second->total / 1e6);
			}
		}
	}
	catch (const profit::exception &e) {
		std::cerr << "Error: " << e.what() << std::endl;
		return 1;
	}
	catch (const std::exception &e) {
		std::cerr << "Error: " << e.what() << std::endl;
		return 1;
	}
	return 0;
}
