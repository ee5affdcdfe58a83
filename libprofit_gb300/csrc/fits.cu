// FITS images on either side of the path (host code only, no device work):
// the PSFs a caller reads in and the model images it writes out, in the
// reference's format (src/fits_utils.cpp: from_fits 60-126, to_fits 150-205).
//
// The file is one primary HDU: 80-byte header cards padded to the 2880-byte
// FITS block, then the pixels as big-endian IEEE doubles, row-major with
// NAXIS1 (the width) fastest, padded with zero bytes to the block. The cards,
// their formatting and the padding rule are the reference's, so that both
// read each other's files and a written file is byte-for-byte the
// reference's: the padding after the header and after the data is always
// 2880 - (length mod 2880) bytes, a whole block when the length is already a
// multiple, and the reader skips the same amount after the END card.
// Byte order is converted with shifts, independently of the host's.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pf_cuda.h"

namespace pf {
void set_last_error(const std::string &msg);
}

namespace {

constexpr size_t kCard = 80;
constexpr size_t kBlock = 36 * kCard;

pf_status invalid_file(const std::string &msg)
{
	pf::set_last_error(msg);
	return PF_ERR_INVALID_FILE;
}

size_t pad_after(size_t length) { return kBlock - length % kBlock; }

void put_be64(double v, unsigned char *out)
{
	uint64_t u;
	std::memcpy(&u, &v, sizeof u);
	for (int i = 0; i < 8; i++) out[i] = (unsigned char)(u >> (56 - 8 * i));
}

double get_be64(const unsigned char *in)
{
	uint64_t u = 0;
	for (int i = 0; i < 8; i++) u = (u << 8) | in[i];
	double v;
	std::memcpy(&v, &u, sizeof v);
	return v;
}

// One card: the text left-justified and blank-filled to 80 columns.
void add_card(std::string &hdr, const char *text)
{
	char c[kCard + 1];
	std::snprintf(c, sizeof c, "%-80s", text);
	hdr.append(c, kCard);
}

struct FileCloser {
	FILE *f;
	~FileCloser()
	{
		if (f) std::fclose(f);
	}
};

struct Header {
	uint32_t width = 0, height = 0;
	double scale_x = 1, scale_y = 1;
	size_t data_offset = 0;
};

// Reads cards up to END and takes the four keys the reference reads
// (matched on the card's first characters, values by the same scanf forms).
pf_status read_header(FILE *f, const std::string &name, Header &h)
{
	char card[kCard + 1];
	size_t consumed = 0;
	while (true) {
		if (std::fread(card, 1, kCard, f) != kCard) {
			return invalid_file("File " + name + " does not look like a normal fits file");
		}
		card[kCard] = '\0';
		consumed += kCard;
		unsigned int u;
		double d;
		if (!std::strncmp(card, "NAXIS1", 6)) {
			if (std::sscanf(card, "NAXIS1 = %u", &u) == 1) h.width = u;
		}
		else if (!std::strncmp(card, "NAXIS2", 6)) {
			if (std::sscanf(card, "NAXIS2 = %u", &u) == 1) h.height = u;
		}
		else if (!std::strncmp(card, "CDELT1", 6)) {
			if (std::sscanf(card, "CDELT1 = %lf", &d) == 1) h.scale_x = d;
		}
		else if (!std::strncmp(card, "CDELT2", 6)) {
			if (std::sscanf(card, "CDELT2 = %lf", &d) == 1) h.scale_y = d;
		}
		else if (!std::strncmp(card, "END", 3)) {
			break;
		}
	}
	h.data_offset = consumed + pad_after(consumed);
	return PF_OK;
}

}  // namespace

extern "C" pf_status pf_fits_read(const char *filename, double *image, size_t image_len, uint32_t *width,
                                  uint32_t *height, double *scale_x, double *scale_y)
{
	if (!filename) {
		pf::set_last_error("pf_fits_read: filename is NULL");
		return PF_ERR_INVALID_PARAMETER;
	}
	const std::string name(filename);
	FileCloser fc{std::fopen(filename, "rb")};
	if (!fc.f) {
		return invalid_file("Couldn't open '" + name + "' for reading: " + std::strerror(errno));
	}
	Header h;
	pf_status s = read_header(fc.f, name, h);
	if (s != PF_OK) return s;
	if (width) *width = h.width;
	if (height) *height = h.height;
	if (scale_x) *scale_x = h.scale_x;
	if (scale_y) *scale_y = h.scale_y;
	if (!image) return PF_OK;
	const uint64_t n = (uint64_t)h.width * h.height;
	if (image_len < n) {
		pf::set_last_error("pf_fits_read: image buffer holds " + std::to_string(image_len) + " values, the file " +
		                   std::to_string(n));
		return PF_ERR_INVALID_PARAMETER;
	}
	const auto less_data = [] {
		return invalid_file("Error while reading file: less data found than expected");
	};
	if (std::fseek(fc.f, (long)h.data_offset, SEEK_SET) != 0) return less_data();
	std::vector<unsigned char> buf(1 << 16);
	uint64_t done = 0;
	while (done < n) {
		const size_t take = (size_t)std::min<uint64_t>(n - done, buf.size() / 8);
		if (std::fread(buf.data(), 8, take, fc.f) != take) return less_data();
		for (size_t i = 0; i < take; i++) image[done + i] = get_be64(buf.data() + 8 * i);
		done += take;
	}
	return PF_OK;
}

extern "C" pf_status pf_fits_write(const char *filename, const double *image, uint32_t width, uint32_t height,
                                   uint32_t offset_x, uint32_t offset_y, double scale_x, double scale_y)
{
	if (!filename || (!image && (uint64_t)width * height > 0)) {
		pf::set_last_error("pf_fits_write: NULL filename or image");
		return PF_ERR_INVALID_PARAMETER;
	}
	std::string name(filename);
	const size_t len = name.size();
	if (len <= 5 || name.compare(len - 5, 5, ".fits") != 0) name += ".fits";
	FileCloser fc{std::fopen(name.c_str(), "wb")};
	if (!fc.f) {
		return invalid_file("Couldn't open '" + name + "' for writing: " + std::strerror(errno));
	}
	// the mandatory keys in fixed format (values right-justified to column 30)
	std::string hdr;
	char text[kCard + 1];
	add_card(hdr, "SIMPLE  =                    T / File conforms to FITS standard");
	add_card(hdr, "BITPIX  =                  -64 / Bits per pixel");
	add_card(hdr, "NAXIS   =                    2 / Number of axes");
	std::snprintf(text, sizeof text, "NAXIS1  =           %10.0u / Width", (unsigned int)width);
	add_card(hdr, text);
	std::snprintf(text, sizeof text, "NAXIS2  =           %10.0u / Height", (unsigned int)height);
	add_card(hdr, text);
	// the world coordinates of pixel (1, 1)'s centre on each axis
	const double crval[2] = {(0.5 - (double)offset_x) * scale_x, (0.5 - (double)offset_y) * scale_y};
	const double cdelt[2] = {scale_x, scale_y};
	for (int a = 0; a < 2; a++) {
		std::snprintf(text, sizeof text, "CRPIX%d  = 1", a + 1);
		add_card(hdr, text);
		std::snprintf(text, sizeof text, "CRVAL%d  = %f", a + 1, crval[a]);
		add_card(hdr, text);
		std::snprintf(text, sizeof text, "CDELT%d  = %f", a + 1, cdelt[a]);
		add_card(hdr, text);
		std::snprintf(text, sizeof text, "CTYPE%d  = ' '", a + 1);
		add_card(hdr, text);
		std::snprintf(text, sizeof text, "CUNIT%d  = ' '", a + 1);
		add_card(hdr, text);
	}
	add_card(hdr, "END");
	hdr.append(pad_after(hdr.size()), ' ');
	bool ok = std::fwrite(hdr.data(), 1, hdr.size(), fc.f) == hdr.size();
	const uint64_t n = (uint64_t)width * height;
	std::vector<unsigned char> buf(1 << 16);
	for (uint64_t done = 0; ok && done < n;) {
		const size_t take = (size_t)std::min<uint64_t>(n - done, buf.size() / 8);
		for (size_t i = 0; i < take; i++) put_be64(image[done + i], buf.data() + 8 * i);
		ok = std::fwrite(buf.data(), 8, take, fc.f) == take;
		done += take;
	}
	if (ok) {
		const std::vector<unsigned char> zeros(pad_after((size_t)(8 * n)), 0);
		ok = std::fwrite(zeros.data(), 1, zeros.size(), fc.f) == zeros.size();
	}
	if (std::fclose(fc.f) != 0) ok = false;
	fc.f = nullptr;
	if (!ok) return invalid_file("Error while writing file '" + name + "': " + std::strerror(errno));
	return PF_OK;
}
