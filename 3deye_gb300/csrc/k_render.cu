// k_render.cu -- Generate_Image (common/src/opencl_wrappers.cpp:967-992):
// grey Lambertian shading of a vertex/normal map into an RGB8 image, for
// visual regression pictures of the model.  The reference's kernel
// (generate_image, named at common/inc/constants.h:170) is not in its
// sources; its arguments -- vertex map, normal map, image size, a
// light_source {point_3f pos; int number} (types/light_source.h:4-8), the
// output image -- are those of the published KinectFusion image generator,
// restated here: per pixel with a valid vertex v and normal n,
//   w  = product over the lights of |dot(normalize(light - v), n)|
//   br = clamp(trunc(205 * w) + 50, 0, 255),  pixel = (br, br, br);
// an invalid pixel is black.  light_source holds one position, so `number`
// is 0 (w = 1) or 1.  Every float operation is a correctly rounded
// intrinsic, so the image equals a C restatement byte for byte.
#include "tde_common.cuh"
#include "tde_launch.cuh"

namespace tde {
namespace {

__global__ void __launch_bounds__(256) generate_image_kernel(const float *__restrict__ vmap,
                                                             const float *__restrict__ nmap, int npix,
                                                             tde_point3f light, int nlights,
                                                             const float *__restrict__ light_dev,
                                                             uint8_t *__restrict__ image) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const float vx = vmap[3 * i], nx = nmap[3 * i];
    int br = 0;
    if (!isnan(vx) && !isnan(nx)) {
        float w = 1.f;
        if (nlights > 0) {
            const float vy = vmap[3 * i + 1], vz = vmap[3 * i + 2];
            const float ny = nmap[3 * i + 1], nz = nmap[3 * i + 2];
            const float lx = light_dev ? light_dev[0] : light.x, ly = light_dev ? light_dev[1] : light.y,
                        lz = light_dev ? light_dev[2] : light.z;
            float dx = __fsub_rn(lx, vx), dy = __fsub_rn(ly, vy), dz = __fsub_rn(lz, vz);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            if (d2 > 0.f) {
                const float inv = __fdiv_rn(1.f, __fsqrt_rn(d2));
                dx = __fmul_rn(dx, inv); dy = __fmul_rn(dy, inv); dz = __fmul_rn(dz, inv);
                w = fabsf(__fadd_rn(__fadd_rn(__fmul_rn(dx, nx), __fmul_rn(dy, ny)), __fmul_rn(dz, nz)));
            } else {
                w = 0.f;  // the light on the surface point: no direction
            }
        }
        if (isnan(w)) w = 0.f;  // a NaN in y or z of an otherwise valid pixel
        else if (w > 2.f) w = 2.f;  // non-unit normals: 255 either way, no int overflow
        br = min(255, max(0, __float2int_rz(__fmul_rn(205.f, w)) + 50));
    }
    const uint8_t b = (uint8_t)br;
    image[3 * i] = b;
    image[3 * i + 1] = b;
    image[3 * i + 2] = b;
}

}  // namespace

int launch_generate_image(const float *vmap, const float *nmap, int W, int H, const tde_point3f &light, int nlights,
                          const float *light_dev, uint8_t *image, cudaStream_t stream) {
    const int npix = W * H;
    if (npix <= 0) return TDE_OK;
    generate_image_kernel<<<div_up((unsigned)npix, 256u), 256, 0, stream>>>(vmap, nmap, npix, light, nlights,
                                                                          light_dev, image);
    return check_launch("generate_image");
}

}  // namespace tde
