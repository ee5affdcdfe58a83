// Direct convolution on the CUDA cores (conv.cuh): the host-side sizing of its
// block shapes and the launches, which take a kernel with the PSF row stride
// compiled in (conv_k*.cu) where every model of the launch shares that stride
// and the kernel reading it per model otherwise.
//
// Measured with a 25 x 25 PSF (stride 28) on the 1024-model step: the stride
// read per model leaves the inner loop with about 34 integer instructions of
// shared-memory addressing per 128 multiply-adds (ncu opcode counters: LEA,
// VIADD, IMAD, IADD3 at 17 % of the forward kernel's instructions, ISETP and
// BRA at 6 %); with it compiled in, the reads are immediate offsets.
#include "conv.cuh"

namespace pf {

PF_CONV_FIXED_ALL(PF_CONV_FIXED_DECL)

template <typename T>
cudaError_t conv_configure(size_t smem, int shape, int kwp);
template <typename T>
void launch_conv(int mode, int shape, int kwp, const ModelDev *models, int n_models, const T *psf, const T *in,
                 const T *direct, T *out, const long long *tile_base, long long n_tiles, size_t smem, int n_sm,
                 cudaStream_t stream);

template <typename T>
int conv_num_shapes()
{
	return std::is_same<T, double>::value ? 1 : 5;
}

template <typename T>
long long conv_tiles(unsigned int w, unsigned int h, int shape)
{
	const Shape sh = shape_of(std::is_same<T, double>::value, shape);
	const unsigned int bw = sh.tx * sh.c, bh = sh.ty * sh.r;
	return (long long)((w + bw - 1) / bw) * ((h + bh - 1) / bh);
}

template <typename T>
size_t conv_smem(unsigned int kw, unsigned int kh, int shape)
{
	const Shape sh = shape_of(std::is_same<T, double>::value, shape);
	const size_t bw = sh.tx * sh.c, bh = sh.ty * sh.r;
	const size_t kwp = (kw + 3) & ~3u;
	return sizeof(T) * ((bw + kwp) * (bh + kh - 1) + kwp * kh);
}

// True if single-precision kernels with PSF row stride kwp are compiled in
bool conv_stride_fixed(int kwp)
{
#define PF_CONV_IS(K) || kwp == K
	return false PF_CONV_FIXED_ALL(PF_CONV_IS);
#undef PF_CONV_IS
}

template <>
cudaError_t conv_configure<float>(size_t smem, int shape, int kwp)
{
#define PF_CONV_CFG(K) \
	if (kwp == K) return conv_configure_f##K(smem, shape);
	PF_CONV_FIXED_ALL(PF_CONV_CFG)
#undef PF_CONV_CFG
	return configure_kernels<float, 0>(smem, shape);
}

template <>
cudaError_t conv_configure<double>(size_t smem, int shape, int)
{
	return configure_kernels<double, 0>(smem, shape);
}

template <>
void launch_conv<float>(int mode, int shape, int kwp, const ModelDev *models, int n_models, const float *psf,
                        const float *in, const float *direct, float *out, const long long *tile_base, long long n_tiles,
                        size_t smem, int n_sm, cudaStream_t stream)
{
#define PF_CONV_RUN(K)                                                                                         \
	if (kwp == K) {                                                                                            \
		launch_conv_f##K(mode, shape, models, n_models, psf, in, direct, out, tile_base, n_tiles, smem, n_sm, stream); \
		return;                                                                                                \
	}
	PF_CONV_FIXED_ALL(PF_CONV_RUN)
#undef PF_CONV_RUN
	launch_kernels<float, 0>(mode, shape, models, n_models, psf, in, direct, out, tile_base, n_tiles, smem, n_sm, stream);
}

template <>
void launch_conv<double>(int mode, int shape, int, const ModelDev *models, int n_models, const double *psf,
                         const double *in, const double *direct, double *out, const long long *tile_base,
                         long long n_tiles, size_t smem, int n_sm, cudaStream_t stream)
{
	launch_kernels<double, 0>(mode, shape, models, n_models, psf, in, direct, out, tile_base, n_tiles, smem, n_sm,
	                          stream);
}

template <typename T>
void conv_tile_dims(int shape, int *bw, int *bh)
{
	const Shape sh = shape_of(std::is_same<T, double>::value, shape);
	*bw = sh.tx * sh.c;
	*bh = sh.ty * sh.r;
}

template void conv_tile_dims<float>(int, int *, int *);
template void conv_tile_dims<double>(int, int *, int *);
template int conv_num_shapes<float>();
template int conv_num_shapes<double>();
template long long conv_tiles<float>(unsigned int, unsigned int, int);
template long long conv_tiles<double>(unsigned int, unsigned int, int);
template size_t conv_smem<float>(unsigned int, unsigned int, int);
template size_t conv_smem<double>(unsigned int, unsigned int, int);

}  // namespace pf
