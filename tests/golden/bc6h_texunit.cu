// BC6H decoding by the GPU's texture unit (test infrastructure): the reference samples its
// BC6H cube map through the graphics hardware (texture.rs:89-94, pathtracing.wgsl:168), so the
// texture unit's decode is the reference decoder against which the CPU oracle (oracle/bc6h.cpp)
// and the library's device decoder are checked.
//
// The blocks go into a CUDA array of 32-bit x 4 elements, one element per 4x4 block, which a
// resource view reads as BC6H (cudaResViewFormat{Unsigned,Signed}BlockCompressed6H, four times
// the array's width and height, as the CUDA runtime documents for block-compressed views); each
// texel is point-sampled at its centre.
#include <cstdint>
#include <cstdio>

#include <cuda_runtime.h>

__global__ void k_texunit_fetch(cudaTextureObject_t tex, int width, int height, float4* out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= width || y >= height) return;
  out[(size_t)y * width + x] = tex2D<float4>(tex, x + 0.5f, y + 0.5f);
}

#define CHECK(call)                                                          \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      std::snprintf(err, err_len, "%s: %s", #call, cudaGetErrorString(e_)); \
      status = 1;                                                            \
      goto done;                                                             \
    }                                                                        \
  } while (0)

// width and height: multiples of 4; blocks: (height / 4) x (width / 4) blocks, row-major;
// out: height x width RGBA32F texels.  Returns 0, or 1 with a message in err.
extern "C" int texunit_bc6h_decode(const void* blocks, int width, int height, int is_signed, float* out, char* err,
                                   int err_len) {
  int status = 0;
  const int bw = width / 4, bh = height / 4;
  cudaArray_t arr = nullptr;
  cudaTextureObject_t tex = 0;
  float4* d_out = nullptr;
  cudaChannelFormatDesc desc = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindUnsigned);
  cudaResourceDesc res = {};
  cudaTextureDesc td = {};
  cudaResourceViewDesc view = {};
  if (width <= 0 || height <= 0 || width % 4 || height % 4) {
    std::snprintf(err, err_len, "size %d x %d is not a positive multiple of 4", width, height);
    return 1;
  }
  CHECK(cudaMallocArray(&arr, &desc, bw, bh));
  CHECK(cudaMemcpy2DToArray(arr, 0, 0, blocks, (size_t)bw * 16, (size_t)bw * 16, bh, cudaMemcpyHostToDevice));
  res.resType = cudaResourceTypeArray;
  res.res.array.array = arr;
  td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModePoint;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 0;
  view.format = is_signed ? cudaResViewFormatSignedBlockCompressed6H : cudaResViewFormatUnsignedBlockCompressed6H;
  view.width = (size_t)width;
  view.height = (size_t)height;
  view.depth = 0;
  CHECK(cudaCreateTextureObject(&tex, &res, &td, &view));
  CHECK(cudaMalloc(&d_out, (size_t)width * height * sizeof(float4)));
  k_texunit_fetch<<<dim3((width + 127) / 128, height), 128>>>(tex, width, height, d_out);
  CHECK(cudaGetLastError());
  CHECK(cudaMemcpy(out, d_out, (size_t)width * height * sizeof(float4), cudaMemcpyDeviceToHost));
done:
  if (tex) cudaDestroyTextureObject(tex);
  if (d_out) cudaFree(d_out);
  if (arr) cudaFreeArray(arr);
  return status;
}
