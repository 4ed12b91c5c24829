// gpe_output.cu - the reference's two field outputs, made from device-side
// downsampling of a field already in HBM:
//   * a density volume, one 16-bit value per block over the padded block grid,
//     written as a MetaImage .mhd/.raw pair (koodit/GrossPitaevskii/
//     GPUGrossPitaevskii_BCC.cu:38-67 and :443-468);
//   * a colour slice of one block plane, written as a 24-bit BMP
//     (GPUGrossPitaevskii_BCC.cu:424-441, jukan_koodit/Output/Picture.cpp:81-129).
// The per-block and per-pixel arithmetic is the reference's, in FP64 with the
// same rounded operations, so the files are byte-identical to its outputs.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "gpe_internal.h"

namespace gpe {
namespace {

// sum over the block's values of |psi|^2 (or, as the reference's loop does, 12
// times |psi_0|^2), times unit, clamped to 65535, truncated to uint16.
template <typename T>
__global__ void volume_kernel(const InstDev *__restrict__ insts, int ii, const T *__restrict__ f, double unit,
                              int quirk, uint16_t *__restrict__ out)
{
    const InstDev &d = insts[ii];
    const int dx = d.nx + 2, dy = d.ny + 2, dz = d.nz + 2;
    const long long total = (long long)dx * dy * dz;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < total;
         v += (long long)gridDim.x * blockDim.x) {
        const int i = int(v % dx);
        const int j = int((v / dx) % dy);
        const int k = int(v / ((long long)dx * dy));
        double sum = 0.0;
        if (i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && k >= 1 && k <= d.nz) {
            for (int l = 0; l < d.slots; l++) {
                const long long o = field_index(d, quirk ? 0 : l, i - 1, j - 1, k - 1);
                const double x = double(f[2 * o]), y = double(f[2 * o + 1]);
                sum = __dadd_rn(sum, __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
            }
            if (quirk)  // the reference adds slot 0's density once per value of the block
                for (int l = d.slots; l < 12; l++) {
                    const long long o = field_index(d, 0, i - 1, j - 1, k - 1);
                    const double x = double(f[2 * o]), y = double(f[2 * o + 1]);
                    sum = __dadd_rn(sum, __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
                }
        }
        sum = __dmul_rn(sum, unit);
        out[v] = sum > 65535.0 ? uint16_t(65535) : uint16_t(sum);
    }
}

// colour of block plane kpad (padded index) for value `slot`:
// (R, G, B) = 256 * gain * (Re psi, |psi|, Im psi), clamped to [0, 255] with
// values below 1 black, as Picture::save(middle = false) does.
__device__ __forceinline__ uint8_t channel(double c)
{
    return c < 1.0 ? uint8_t(0) : (c > 255.0 ? uint8_t(255) : uint8_t(int(c)));
}

template <typename T>
__global__ void slice_kernel(const InstDev *__restrict__ insts, int ii, const T *__restrict__ f, int kpad, int slot,
                             double gain, uint8_t *__restrict__ rgb)
{
    const InstDev &d = insts[ii];
    const int dx = d.nx + 2, dy = d.ny + 2;
    const int total = dx * dy;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < total; v += gridDim.x * blockDim.x) {
        const int i = v % dx, j = v / dx;
        double x = 0.0, y = 0.0;
        if (i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && kpad >= 1 && kpad <= d.nz) {
            const long long o = field_index(d, slot, i - 1, j - 1, kpad - 1);
            x = double(f[2 * o]);
            y = double(f[2 * o + 1]);
        }
        const double norm = __dsqrt_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)));
        rgb[3 * v + 0] = channel(__dmul_rn(256.0, __dmul_rn(gain, x)));
        rgb[3 * v + 1] = channel(__dmul_rn(256.0, __dmul_rn(gain, norm)));
        rgb[3 * v + 2] = channel(__dmul_rn(256.0, __dmul_rn(gain, y)));
    }
}

}  // namespace

cudaError_t launch_volume(int precision, const InstDev *inst, int ii, const void *field, double unit, int quirk,
                          uint16_t *out, long long total, cudaStream_t s)
{
    long long g = (total + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    if (precision == GPE_FP64)
        volume_kernel<double><<<int(g), 256, 0, s>>>(inst, ii, (const double *)field, unit, quirk, out);
    else
        volume_kernel<float><<<int(g), 256, 0, s>>>(inst, ii, (const float *)field, unit, quirk, out);
    return cudaGetLastError();
}

cudaError_t launch_slice(int precision, const InstDev *inst, int ii, const void *field, int kpad, int slot,
                         double gain, uint8_t *rgb, int total, cudaStream_t s)
{
    const int g = (total + 255) / 256;
    if (precision == GPE_FP64)
        slice_kernel<double><<<g, 256, 0, s>>>(inst, ii, (const double *)field, kpad, slot, gain, rgb);
    else
        slice_kernel<float><<<g, 256, 0, s>>>(inst, ii, (const float *)field, kpad, slot, gain, rgb);
    return cudaGetLastError();
}

}  // namespace gpe

using namespace gpe;

extern "C" {

static gpe_status gpe_write_metaimage_impl(const char *path, const uint16_t *vol, uint32_t dx, uint32_t dy, uint32_t dz,
                                           const double *spacing)
{
    if (!path || !vol || !spacing || !dx || !dy || !dz)
        return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_write_metaimage: bad arguments");
    // saveVolumeMap (GPUGrossPitaevskii_BCC.cu:38-67): raw data in <path>.raw,
    // text header in <path>, numbers in the stream's default 6-digit format.
    const std::string raw = std::string(path) + ".raw";
    FILE *fr = std::fopen(raw.c_str(), "wb");
    if (!fr) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_write_metaimage: cannot write " + raw);
    const size_t n = size_t(dx) * dy * dz;
    const bool ok = std::fwrite(vol, 2, n, fr) == n;
    std::fclose(fr);
    if (!ok) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_write_metaimage: short write " + raw);
    FILE *fh = std::fopen(path, "w");
    if (!fh) return fail(GPE_ERR_INVALID_ARGUMENT, std::string("gpe_write_metaimage: cannot write ") + path);
    std::fprintf(fh, "ObjectType              = Image\n");
    std::fprintf(fh, "NDims                   = 3\n");
    std::fprintf(fh, "BinaryData              = True\n");
    std::fprintf(fh, "CompressedData          = False\n");
    std::fprintf(fh, "BinaryDataByteOrderMSB  = False\n");
    std::fprintf(fh, "TransformMatrix         = 1 0 0 0 1 0 0 0 1\n");
    std::fprintf(fh, "Offset                  = %g %g %g\n", -0.5 * dx * spacing[0], -0.5 * dy * spacing[1],
                 -0.5 * dz * spacing[2]);
    std::fprintf(fh, "CenterOfRotation        = 0 0 0\n");
    std::fprintf(fh, "DimSize                 = %u %u %u\n", dx, dy, dz);
    std::fprintf(fh, "ElementSpacing          = %g %g %g\n", spacing[0], spacing[1], spacing[2]);
    std::fprintf(fh, "ElementNumberOfChannels = 1\n");
    std::fprintf(fh, "ElementType             = MET_USHORT\n");
    std::fprintf(fh, "ElementDataFile         = %s\n", raw.c_str());
    std::fclose(fh);
    return GPE_OK;
}

gpe_status gpe_write_metaimage(const char *path, const uint16_t *vol, uint32_t dx, uint32_t dy, uint32_t dz,
                               const double *spacing)
{
    GPE_GUARD(gpe_write_metaimage_impl(path, vol, dx, dy, dz, spacing));
}

static gpe_status gpe_write_bmp_impl(const char *path, const uint8_t *rgb, uint32_t width, uint32_t height)
{
    if (!path || !rgb || !width || !height) return fail(GPE_ERR_INVALID_ARGUMENT, "gpe_write_bmp: bad arguments");
    // Picture::save (jukan_koodit/Output/Picture.cpp:81-129): 24-bit, bottom-up
    // rows of (B, G, R) padded to 4 bytes; its header states 4 bytes per pixel.
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return fail(GPE_ERR_INVALID_ARGUMENT, std::string("gpe_write_bmp: cannot write ") + path);
    const uint32_t offs = 14 + 40, data = 4 * width * height, size = offs + data, zero = 0, header = 40;
    const uint16_t one = 1, bits = 24;
    std::fwrite("BM", 1, 2, fp);
    std::fwrite(&size, 4, 1, fp);
    std::fwrite(&zero, 4, 1, fp);
    std::fwrite(&offs, 4, 1, fp);
    std::fwrite(&header, 4, 1, fp);
    std::fwrite(&width, 4, 1, fp);
    std::fwrite(&height, 4, 1, fp);
    std::fwrite(&one, 2, 1, fp);
    std::fwrite(&bits, 2, 1, fp);
    std::fwrite(&zero, 4, 1, fp);
    std::fwrite(&data, 4, 1, fp);
    for (int k = 0; k < 4; k++) std::fwrite(&zero, 4, 1, fp);
    const uint32_t rowend = 3 - ((3 * width + 3) % 4);
    for (uint32_t y = 0; y < height; y++) {
        for (uint32_t x = 0; x < width; x++) {
            const uint8_t *p = rgb + 3 * (size_t(y) * width + x);
            const uint8_t bgr[3] = {p[2], p[1], p[0]};
            std::fwrite(bgr, 1, 3, fp);
        }
        if (rowend > 0) std::fwrite(&zero, 1, rowend, fp);
    }
    std::fclose(fp);
    return GPE_OK;
}

gpe_status gpe_write_bmp(const char *path, const uint8_t *rgb, uint32_t width, uint32_t height)
{
    GPE_GUARD(gpe_write_bmp_impl(path, rgb, width, height));
}

}  // extern "C"
