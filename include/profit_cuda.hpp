/*
 * profit_cuda.hpp - C++ host interface of the GB300 backend, mirroring the
 * part of libprofit's public C++ API that drives image generation, over the
 * C ABI of pf_cuda.h. Header-only; link against libpfcuda.so.
 *
 *   profit::Model                 -> profit_cuda::Model       (include/profit/model.h:60-408)
 *   Model::add_profile            -> Model::add_profile       (src/model.cpp:103-135)
 *   Profile::parameter            -> Profile::parameter       (src/profile.cpp:84-163)
 *   Model::evaluate               -> Model::evaluate          (src/model.cpp:259-320)
 *   get_opencl_environment        -> get_cuda_environment     (include/profit/opencl.h:159-168)
 *   Model::set_opencl_env         -> Model::set_cuda_env      (include/profit/model.h:305-311)
 *   create_convolver(type, prefs) -> create_convolver("cuda") (src/convolve.cpp:521-584)
 *   Convolver::convolve           -> Convolver::convolve      (include/profit/convolve.h:98-99)
 *   from_fits, to_fits            -> from_fits, to_fits       (src/fits_utils.cpp:60-205)
 *   invalid_parameter, unknown_parameter, opencl_error, invalid_file
 *                                 -> invalid_parameter, unknown_parameter, cuda_error, invalid_file
 *                                    (include/profit/exceptions.h:41-104,
 *                                    include/profit/fits_utils.h:34-43)
 * Parameter names, types, defaults and validation messages are the
 * reference's; errors become exceptions of the same categories.
 */
#ifndef PROFIT_CUDA_HPP
#define PROFIT_CUDA_HPP

#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "pf_cuda.h"

namespace profit_cuda {

class exception : public std::exception {
public:
	explicit exception(const std::string &what) : m_what(what) {}
	const char *what() const noexcept override { return m_what.c_str(); }

private:
	std::string m_what;
};

class invalid_parameter : public exception {
public:
	explicit invalid_parameter(const std::string &what) : exception(what) {}
};

class unknown_parameter : public exception {
public:
	explicit unknown_parameter(const std::string &what) : exception(what) {}
};

class cuda_error : public exception {
public:
	explicit cuda_error(const std::string &what) : exception(what) {}
};

class invalid_file : public exception {
public:
	explicit invalid_file(const std::string &what) : exception(what) {}
};

inline void check(pf_status s)
{
	if (s == PF_OK) return;
	const std::string msg = pf_last_error();
	if (s == PF_ERR_INVALID_PARAMETER) throw invalid_parameter(msg);
	if (s == PF_ERR_UNKNOWN_PARAMETER) throw unknown_parameter(msg);
	if (s == PF_ERR_CUDA || s == PF_ERR_NO_MEMORY) throw cuda_error(msg);
	if (s == PF_ERR_INVALID_FILE) throw invalid_file(msg);
	throw exception(msg);
}

/* A 2-D image: row-major doubles, element (x, y) at x + y * width
 * (include/profit/image.h:664-823). */
class Image {
public:
	Image() : m_w(0), m_h(0) {}
	Image(unsigned int w, unsigned int h) : m_data((size_t)w * h, 0.0), m_w(w), m_h(h) {}
	Image(std::vector<double> data, unsigned int w, unsigned int h) : m_data(std::move(data)), m_w(w), m_h(h)
	{
		if (m_data.size() != (size_t)w * h) throw std::invalid_argument("data.size() != w * h");
	}
	unsigned int getWidth() const { return m_w; }
	unsigned int getHeight() const { return m_h; }
	size_t size() const { return m_data.size(); }
	double *data() { return m_data.data(); }
	const double *data() const { return m_data.data(); }
	double &operator[](size_t i) { return m_data[i]; }
	double operator[](size_t i) const { return m_data[i]; }
	double total() const
	{
		double s = 0;
		for (double v : m_data) s += v;
		return s;
	}

private:
	std::vector<double> m_data;
	unsigned int m_w, m_h;
};

/* A CUDA environment (OpenCLEnv analogue). use_double selects the plain FP64
 * path that reproduces the reference's arithmetic; profile, the stage timing
 * and counts of Model::get_stats. */
class CUDAEnv {
public:
	CUDAEnv(int device, bool use_double, bool profile = false) : m_env(nullptr)
	{
		check(pf_env_create(device, (use_double ? PF_ENV_DOUBLE : 0u) | (profile ? PF_ENV_PROFILE : 0u), &m_env));
	}
	~CUDAEnv() { pf_env_destroy(m_env); }
	CUDAEnv(const CUDAEnv &) = delete;
	CUDAEnv &operator=(const CUDAEnv &) = delete;
	pf_env *get() const { return m_env; }

private:
	pf_env *m_env;
};
typedef std::shared_ptr<CUDAEnv> CUDAEnvPtr;

inline CUDAEnvPtr get_cuda_environment(int device = 0, bool use_double = true, bool profile = false)
{
	return std::make_shared<CUDAEnv>(device, use_double, profile);
}

class Model;

/* Model::get_stats (include/profit/profile.h:46-73, src/model.cpp:362-368),
 * for an environment with PF_ENV_PROFILE (CUDAEnv(device, use_double,
 * profile = true)). This backend evaluates all of a model's profiles in fused
 * passes timed as a whole: cuda_times holds those passes' device times, and
 * `total` the profile's share -- the setup pass split evenly, the evaluation
 * pass by the profile's evaluate_at calls. */
typedef long long nsecs_t;
struct CUDA_times {
	nsecs_t setup = 0, evaluation = 0, convolution = 0;
};
class ProfileStats {
public:
	virtual ~ProfileStats() {}
	nsecs_t total = 0;
};
struct RadialProfileStats : ProfileStats {
	CUDA_times cuda_times;
	unsigned long long evaluations = 0;        // evaluate_at calls
	std::map<int, unsigned long long> integrations;  // subsample_pixel calls per recursion level
};

/* A profile of a Model (include/profit/profile.h:78-260). */
class Profile {
public:
	Profile(const std::string &name, int kind) : m_name(name)
	{
		m_desc = pf_profile_desc();
		m_desc.kind = kind;
		m_desc.convolve = 0;
		m_desc.rough = 0;
		m_desc.adjust = 1;
		m_desc.rescale_flux = 0;
		m_desc.resolution = 9;
		m_desc.max_recursions = 2;
		m_desc.acc = kind == PF_FERRER ? 1.0 : 0.1;
		m_desc.rscale_switch = 1.0;
		m_desc.rscale_max = 0.0;
		for (int i = 0; i < PF_NPAR; i++) m_desc.par[i] = 0.0;
		if (is_radial()) {
			m_desc.par[PF_P_MAG] = 15.0;
			m_desc.par[PF_P_AXRAT] = 1.0;
		}
		// constructor defaults of each profile
		switch (kind) {
		case PF_SERSIC: set_slots({1.0, 1.0}); break;
		case PF_CORESERSIC: set_slots({1.0, 4.0, 1.0, 1.0, 1.0}); break;
		case PF_MOFFAT: set_slots({3.0, 2.0}); break;
		case PF_USER: {
			const double *defaults = nullptr;
			uint32_t count = 0;
			if (pf_user_profile_info(nullptr, nullptr, &defaults, &count) == PF_OK) {
				for (uint32_t i = 0; i < count; i++) m_desc.par[PF_P_X0 + i] = defaults[i];
			}
			break;
		}
		case PF_FERRER: set_slots({3.0, 1.0, 1.0}); break;
		case PF_KING: set_slots({1.0, 3.0, 2.0}); break;
		case PF_BROKENEXP: set_slots({1.0, 1.0, 1.0, 1.0}); break;
		default: break;
		}
	}

	const std::string &get_name() const { return m_name; }
	const pf_profile_desc &desc() const { return m_desc; }

	void parameter(const std::string &name, double value)
	{
		double *slot = double_slot(name);
		if (!slot) throw invalid_parameter("Unknown double parameter in profile " + m_name + ": " + name);
		*slot = value;
	}
	void parameter(const std::string &name, bool value)
	{
		int32_t *slot = bool_slot(name);
		if (!slot) throw invalid_parameter("Unknown bool parameter in profile " + m_name + ": " + name);
		*slot = value ? 1 : 0;
	}
	void parameter(const std::string &name, unsigned int value)
	{
		uint32_t *slot = uint_slot(name);
		if (!slot) throw invalid_parameter("Unknown unsigned int parameter in profile " + m_name + ": " + name);
		*slot = value;
	}
	/* "name=value" */
	void parameter(const std::string &spec)
	{
		const size_t eq = spec.find('=');
		if (eq == std::string::npos || spec.find('=', eq + 1) != std::string::npos) {
			throw invalid_parameter("missing = in parameter: " + spec);
		}
		const std::string name = trim(spec.substr(0, eq)), val = trim(spec.substr(eq + 1));
		try {
			if (int32_t *b = bool_slot(name)) {
				*b = std::stoul(val, nullptr, 10) != 0;
				return;
			}
			if (uint32_t *u = uint_slot(name)) {
				*u = (uint32_t)std::stoul(val, nullptr, 10);
				return;
			}
			if (double *d = double_slot(name)) {
				*d = std::stod(val);
				return;
			}
		}
		catch (const std::logic_error &) {
		}
		throw unknown_parameter("Profile " + m_name + " doesn't support parameter " + name +
		                        ", or parameter has invalid value: " + val);
	}

private:
	bool is_radial() const
	{
		return (m_desc.kind >= PF_SERSIC && m_desc.kind <= PF_BROKENEXP) || m_desc.kind == PF_USER;
	}

	void set_slots(std::initializer_list<double> vals)
	{
		int i = PF_P_X0;
		for (double v : vals) m_desc.par[i++] = v;
	}

	static std::string trim(const std::string &s)
	{
		const size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
		return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
	}

	int32_t *bool_slot(const std::string &n)
	{
		if (n == "convolve") return &m_desc.convolve;
		if (is_radial() && n == "rough") return &m_desc.rough;
		if (is_radial() && n == "adjust") return &m_desc.adjust;
		if (is_radial() && n == "force_cpu") return &m_force_cpu;  // accepted; there is no CPU path here
		if (m_desc.kind == PF_SERSIC && n == "rescale_flux") return &m_desc.rescale_flux;
		return nullptr;
	}

	uint32_t *uint_slot(const std::string &n)
	{
		if (is_radial() && n == "resolution") return &m_desc.resolution;
		if (is_radial() && n == "max_recursions") return &m_desc.max_recursions;
		return nullptr;
	}

	double *double_slot(const std::string &n)
	{
		static const std::map<int, std::vector<std::string>> specific = {
		    {PF_SERSIC, {"re", "nser"}},
		    {PF_CORESERSIC, {"re", "nser", "rb", "a", "b"}},
		    {PF_MOFFAT, {"fwhm", "con"}},
		    {PF_FERRER, {"rout", "a", "b"}},
		    {PF_KING, {"rc", "rt", "a"}},
		    {PF_BROKENEXP, {"h1", "h2", "rb", "a"}},
		    {PF_SKY, {"bg"}},
		};
		static const char *common[] = {"xcen", "ycen", "mag", "ang", "axrat", "box"};
		if (is_radial()) {
			for (int i = 0; i < 6; i++)
				if (n == common[i]) return &m_desc.par[i];
			if (n == "acc") return &m_desc.acc;
			if (n == "rscale_switch") return &m_desc.rscale_switch;
			if (n == "rscale_max") return &m_desc.rscale_max;
		}
		if (m_desc.kind == PF_PSF) {
			for (int i = 0; i < 3; i++)
				if (n == common[i]) return &m_desc.par[i];
		}
		auto it = specific.find(m_desc.kind);
		if (it != specific.end()) {
			for (size_t i = 0; i < it->second.size(); i++)
				if (n == it->second[i]) return &m_desc.par[PF_P_X0 + i];
		}
		if (m_desc.kind == PF_USER) {  // the compiled-in user profile's own parameters
			const char *const *names = nullptr;
			uint32_t count = 0;
			if (pf_user_profile_info(nullptr, &names, nullptr, &count) == PF_OK) {
				for (uint32_t i = 0; i < count; i++)
					if (n == names[i]) return &m_desc.par[PF_P_X0 + i];
			}
		}
		return nullptr;
	}

	std::string m_name;
	pf_profile_desc m_desc;
	int32_t m_force_cpu = 0;
};
typedef std::shared_ptr<Profile> ProfilePtr;

/* Model::evaluate on the GPU. */
class Model {
public:
	Model(unsigned int width = 0, unsigned int height = 0) : m_width(width), m_height(height) {}

	ProfilePtr add_profile(const std::string &name)
	{
		static const std::map<std::string, int> kinds = {
		    {"sersic", PF_SERSIC}, {"coresersic", PF_CORESERSIC}, {"moffat", PF_MOFFAT},
		    {"ferrer", PF_FERRER}, {"ferrers", PF_FERRER},       {"king", PF_KING},
		    {"brokenexp", PF_BROKENEXP}, {"sky", PF_SKY},        {"psf", PF_PSF},
		    {"null", PF_NULL}};
		auto it = kinds.find(name);
		int kind = it == kinds.end() ? -1 : it->second;
		const char *user = nullptr;  // the user-defined profile compiled into the library, if any
		if (kind < 0 && pf_user_profile_info(&user, nullptr, nullptr, nullptr) == PF_OK && name == user) {
			kind = PF_USER;
		}
		if (kind < 0) throw invalid_parameter("Unknown profile name: " + name);
		m_profiles.push_back(std::make_shared<Profile>(name, kind));
		return m_profiles.back();
	}

	void set_dimensions(unsigned int w, unsigned int h) { m_width = w, m_height = h; }
	void set_image_pixel_scale(const std::pair<double, double> &s) { m_scale = s; }
	std::pair<double, double> get_image_pixel_scale() const { return m_scale; }
	bool has_profiles() const { return !m_profiles.empty(); }
	void set_psf_pixel_scale(const std::pair<double, double> &s) { m_psf_scale = s; }
	void set_magzero(double magzero) { m_magzero = magzero; }
	void set_finesampling(unsigned int fs)
	{
		if (fs == 0) throw std::invalid_argument("finesampling must be > 0");
		m_finesampling = fs;
	}
	void set_return_finesampled(bool b) { m_return_finesampled = b; }
	/* The PSF is normalised to unit sum on the device, as set_psf does. */
	void set_psf(const Image &psf) { m_psf = psf; }
	void set_cuda_env(const CUDAEnvPtr &env) { m_env = env; }
	CUDAEnvPtr get_cuda_env() const { return m_env; }
	/* Model::set_mask / set_adjust_mask (include/profit/model.h:219-246): one
	 * byte per pixel, non-zero = evaluate, row-major width x height; the
	 * model's dimensions when adjusted (the default), the drawing dimensions
	 * otherwise. Empty: no mask. */
	void set_mask(const std::vector<uint8_t> &mask, unsigned int width, unsigned int height)
	{
		if (mask.size() != (size_t)width * height) throw invalid_parameter("mask size != width x height");
		m_mask = mask;
		m_mask_w = width;
		m_mask_h = height;
	}
	void set_adjust_mask(bool adjust) { m_adjust_mask = adjust; }
	/* Model::set_crop: the direct convolutions add no padding, so the image
	 * is the cropped one at offset (0, 0); with the FFT convolver (double
	 * precision) crop false keeps its uncropped frame less the PSF padding. */
	void set_crop(bool crop) { m_crop = crop; }
	/* The convolver of create_convolver's string form (src/convolve.cpp:
	 * 562-584) on this backend: "brute" / "cuda" the direct convolution, "fft"
	 * / "cuda-fft" the FFT convolution, "auto" (the default) the library's
	 * choice. */
	void set_convolver(const std::string &type)
	{
		if (type == "brute" || type == "cuda") m_convolver = PF_CONV_BRUTE;
		else if (type == "fft" || type == "cuda-fft") m_convolver = PF_CONV_FFT;
		else if (type == "auto") m_convolver = PF_CONV_AUTO;
		else throw invalid_parameter("Convolver of type " + type + " is not supported");
	}

	/* Model::evaluate(Point &offset_out): the offset of the requested area in
	 * the returned image */
	Image evaluate(std::pair<unsigned int, unsigned int> &offset_out)
	{
		Image img = evaluate();
		pf_model_desc m = desc();
		std::vector<pf_profile_desc> profs;
		for (auto &p : m_profiles) profs.push_back(p->desc());
		uint32_t x = 0, y = 0;
		check(pf_model_output_offset(&m, profs.data(), &x, &y));
		offset_out = {x, y};
		return img;
	}

	Image evaluate()
	{
		if (!m_env) m_env = get_cuda_environment(0, true);
		pf_model_desc m = desc();
		std::vector<pf_profile_desc> profs;
		for (auto &p : m_profiles) profs.push_back(p->desc());
		uint32_t w = 0, h = 0;
		check(pf_model_output_dims(&m, profs.data(), &w, &h));
		Image out(w, h);
		check(pf_model_evaluate_masked(m_env->get(), &m, profs.data(), m_psf.size() ? m_psf.data() : nullptr,
		                               m_mask.empty() ? nullptr : m_mask.data(), out.data(), &w, &h));
		return out;
	}

	/* Model::get_stats: {profile name: stats} of the last evaluate() (keyed
	 * by name as the reference's map: a later profile of the same name
	 * replaces an earlier one); empty without PF_ENV_PROFILE. */
	std::map<std::string, std::shared_ptr<ProfileStats>> get_stats() const
	{
		std::map<std::string, std::shared_ptr<ProfileStats>> out;
		if (!m_env || m_profiles.empty()) return out;
		pf_stage_times t = pf_stage_times();
		std::vector<int64_t> counts(m_profiles.size() * 32, 0);
		check(pf_env_last_model_stats(m_env->get(), &t, counts.data(), m_profiles.size()));
		if (t.forward_calls == 0) return out;
		unsigned long long all = 0;
		for (size_t i = 0; i < m_profiles.size(); i++) all += counts[i * 32 + 30] + counts[i * 32 + 31];
		for (size_t i = 0; i < m_profiles.size(); i++) {
			auto st = std::make_shared<RadialProfileStats>();
			st->cuda_times.setup = (nsecs_t)(t.setup_ms * 1e6);
			st->cuda_times.evaluation = (nsecs_t)(t.eval_ms * 1e6);
			st->cuda_times.convolution = (nsecs_t)(t.finish_ms * 1e6);
			st->evaluations = (unsigned long long)(counts[i * 32 + 30] + counts[i * 32 + 31]);
			for (int l = 0; l < 16; l++) {
				if (counts[i * 32 + l]) st->integrations[l] = (unsigned long long)counts[i * 32 + l];
			}
			const double share = all ? (double)st->evaluations / all : 1.0 / m_profiles.size();
			st->total = (nsecs_t)((t.setup_ms / m_profiles.size() + t.eval_ms * share) * 1e6);
			out[m_profiles[i]->get_name()] = st;
		}
		return out;
	}

	pf_model_desc desc() const
	{
		pf_model_desc m = pf_model_desc();
		m.width = m_width;
		m.height = m_height;
		m.scale_x = m_scale.first;
		m.scale_y = m_scale.second;
		m.magzero = m_magzero;
		m.finesampling = m_finesampling;
		m.return_finesampled = m_return_finesampled ? 1 : 0;
		m.first_profile = 0;
		m.n_profiles = (uint32_t)m_profiles.size();
		m.psf_offset = m_psf.size() ? 0 : -1;
		m.psf_w = m_psf.getWidth();
		m.psf_h = m_psf.getHeight();
		m.psf_scale_x = m_psf_scale.first;
		m.psf_scale_y = m_psf_scale.second;
		m.convolver = m_convolver;
		m.mask_offset = m_mask.empty() ? -1 : 0;
		m.adjust_mask = m_adjust_mask ? 1 : 0;
		m.mask_w = m_mask_w;
		m.mask_h = m_mask_h;
		m.no_crop = m_crop ? 0 : 1;
		return m;
	}

private:
	unsigned int m_width, m_height;
	std::pair<double, double> m_scale{1.0, 1.0}, m_psf_scale{1.0, 1.0};
	double m_magzero = 0.0;
	unsigned int m_finesampling = 1;
	bool m_return_finesampled = true;
	bool m_adjust_mask = true;
	bool m_crop = true;
	int32_t m_convolver = PF_CONV_AUTO;
	std::vector<uint8_t> m_mask;
	unsigned int m_mask_w = 0, m_mask_h = 0;
	Image m_psf;
	CUDAEnvPtr m_env;
	std::vector<ProfilePtr> m_profiles;
};

/* ConvolverType::CUDA: a direct convolution on the GPU with the reference's
 * semantics (Convolver::convolve, src/convolve.cpp:55-99). It adds no
 * padding, so crop = false returns the same image and offset (0, 0);
 * offset_out (x, y) may be null, the reference's NO_OFFSET. */
class Convolver {
public:
	explicit Convolver(CUDAEnvPtr env) : m_env(std::move(env)) {}
	Image convolve(const Image &src, const Image &krn, const std::vector<uint8_t> &mask = {}, bool crop = true,
	               std::pair<unsigned int, unsigned int> *offset_out = nullptr)
	{
		Image out(src.getWidth(), src.getHeight());
		uint32_t ox = 0, oy = 0;
		check(pf_convolve_crop(m_env->get(), src.data(), src.getWidth(), src.getHeight(), krn.data(),
		                       krn.getWidth(), krn.getHeight(), mask.empty() ? nullptr : mask.data(), crop ? 1 : 0,
		                       out.data(), &ox, &oy));
		if (offset_out) *offset_out = {ox, oy};
		return out;
	}

private:
	CUDAEnvPtr m_env;
};
typedef std::shared_ptr<Convolver> ConvolverPtr;

inline ConvolverPtr create_convolver(const std::string &type, CUDAEnvPtr env = nullptr)
{
	if (type != "cuda") throw invalid_parameter("Unsupported convolver type: " + type);
	return std::make_shared<Convolver>(env ? env : get_cuda_environment(0, true));
}

/* The reference's Point (whole pixels) and PixelScale (include/profit/image.h:47-61, 823). */
typedef std::pair<double, double> PixelScale;
struct Point {
	unsigned int x = 0, y = 0;
};

/* profit::from_fits (src/fits_utils.cpp:60-126): the image of a FITS file and
 * its pixel scale (CDELT1, CDELT2). */
inline Image from_fits(const std::string &filename, PixelScale &pixel_scale)
{
	uint32_t w = 0, h = 0;
	double sx = 1, sy = 1;
	check(pf_fits_read(filename.c_str(), nullptr, 0, &w, &h, &sx, &sy));
	Image img(w, h);
	check(pf_fits_read(filename.c_str(), img.data(), img.size(), &w, &h, &sx, &sy));
	pixel_scale = {sx, sy};
	return img;
}

/* profit::to_fits (src/fits_utils.cpp:150-205): ".fits" is appended to the
 * name unless it ends in it. */
inline void to_fits(const Image &image, const Point &offset, const PixelScale &pixel_scale, std::string fname)
{
	check(pf_fits_write(fname.c_str(), image.data(), image.getWidth(), image.getHeight(), offset.x, offset.y,
	                    pixel_scale.first, pixel_scale.second));
}

}  // namespace profit_cuda

#endif /* PROFIT_CUDA_HPP */
