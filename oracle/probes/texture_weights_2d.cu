// Probe of the texture unit's bilinear weights (test infrastructure: it
// measured the rule oracle mode 2 uses, see
// oracle/probes/check_texture_weights.py). Same texture settings as the
// reference PSF texture (normalized coordinates, linear filter, border).
// (1) y-ramp: a 2 x H float texture with T[j][i] = j, fetched at u = 0.25
//     (column 0 exactly) and M values of v: returns j + weight (H = 164, 3495).
// (2) unit texel: a 4 x 4 float texture with T[1][1] = 1, fetched at M random
//     (u, v) around that texel: returns that corner's bilinear weight.
// Usage: texture_weights_2d OUT_DIR -> OUT_DIR/tex_y164.bin, tex_y3495.bin,
// tex_delta.bin, each float2 uv[M] then float fetch[M]. Every access stays
// inside the M-entry buffers.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <random>
#include <string>
#include <cuda_runtime.h>
__global__ void k_fetch2(cudaTextureObject_t t, const float2* uv, float* out, int m)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < m) out[i] = tex2D<float>(t, uv[i].x, uv[i].y);
}
static cudaTextureObject_t make(const std::vector<float>& tab, int W, int H)
{
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    cudaArray_t arr; cudaMallocArray(&arr, &ch, W, H);
    cudaMemcpy2DToArray(arr, 0, 0, tab.data(), W * 4, W * 4, H, cudaMemcpyHostToDevice);
    cudaResourceDesc rd = {}; rd.resType = cudaResourceTypeArray; rd.res.array.array = arr;
    cudaTextureDesc td = {}; td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear; td.readMode = cudaReadModeElementType; td.normalizedCoords = 1;
    cudaTextureObject_t t; cudaCreateTextureObject(&t, &rd, &td, nullptr);
    return t;
}
static int run(cudaTextureObject_t t, const std::vector<float2>& uv, const char* path)
{
    const int M = (int)uv.size();
    std::vector<float> out(M);
    float2* duv; float* dout; cudaMalloc(&duv, M * 8); cudaMalloc(&dout, M * 4);
    cudaMemcpy(duv, uv.data(), M * 8, cudaMemcpyHostToDevice);
    k_fetch2<<<(M + 255) / 256, 256>>>(t, duv, dout, M);
    cudaError_t e = cudaDeviceSynchronize();
    if(e != cudaSuccess) { printf("error %s\n", cudaGetErrorString(e)); return 1; }
    cudaMemcpy(out.data(), dout, M * 4, cudaMemcpyDeviceToHost);
    FILE* f = fopen(path, "wb"); fwrite(uv.data(), 8, M, f); fwrite(out.data(), 4, M, f); fclose(f);
    cudaFree(duv); cudaFree(dout);
    return 0;
}
int main(int argc, char** argv)
{
    if(argc != 2) { printf("usage: %s OUT_DIR\n", argv[0]); return 2; }
    const std::string dir = argv[1];
    const int M = 200003;
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    for(int H : {164, 3495}) {
        std::vector<float> tab(2 * H);
        for(int j = 0; j < H; j++) tab[2 * j] = tab[2 * j + 1] = (float)j;
        std::vector<float2> uv(M);
        for(int k = 0; k < M; k++) uv[k] = make_float2(0.25f, (float)((0.5 + (double)k * (H - 1.0) / (M - 1.0)) / H));
        if(run(make(tab, 2, H), uv, (dir + "/tex_y" + std::to_string(H) + ".bin").c_str())) return 1;
    }
    std::vector<float> tab(16, 0.0f); tab[1 * 4 + 1] = 1.0f;
    std::vector<float2> uv(M);
    for(int k = 0; k < M; k++) uv[k] = make_float2(0.125f + 0.5f * U(rng), 0.125f + 0.5f * U(rng));
    if(run(make(tab, 4, 4), uv, (dir + "/tex_delta.bin").c_str())) return 1;
    printf("ok\n");
    return 0;
}
