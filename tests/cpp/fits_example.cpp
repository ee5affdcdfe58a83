// Reads a FITS image with profit_cuda::from_fits and writes it back with
// profit_cuda::to_fits, as a libprofit program does with profit::from_fits
// and profit::to_fits (include/profit/fits_utils.h:45-49).
//   fits_example <in.fits> <out name> <offset x> <offset y>
// Prints "<width> <height> <scale x> <scale y>" on success.
#include <cstdio>
#include <cstdlib>

#include "profit_cuda.hpp"

int main(int argc, char **argv)
{
	if (argc != 5) return 2;
	try {
		profit_cuda::PixelScale scale;
		profit_cuda::Image img = profit_cuda::from_fits(argv[1], scale);
		profit_cuda::Point offset;
		offset.x = (unsigned int)std::strtoul(argv[3], nullptr, 10);
		offset.y = (unsigned int)std::strtoul(argv[4], nullptr, 10);
		profit_cuda::to_fits(img, offset, scale, argv[2]);
		std::printf("%u %u %.17g %.17g\n", img.getWidth(), img.getHeight(), scale.first, scale.second);
	}
	catch (const profit_cuda::invalid_file &e) {
		std::printf("invalid_file: %s\n", e.what());
		return 1;
	}
	return 0;
}
