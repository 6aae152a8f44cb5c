// Probe of the texture unit's linear-filter weight along one axis (test
// infrastructure: it measured the rule oracle mode 2 uses, see
// oracle/probes/check_texture_weights.py). A W x 1 float texture with
// T[i] = i, so that a fetch between texels i and i + 1 returns i + weight;
// normalized coordinates, linear filter, border addressing (the reference
// PSF texture's settings); M coordinates spread over the texels.
// Usage: texture_weights_1d W M OUT  -> OUT = float u[M], float fetch[M].
// Every access stays inside the M-entry buffers.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>
__global__ void k_fetch(cudaTextureObject_t t, const float* u, float* out, int m, float v)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < m) out[i] = tex2D<float>(t, u[i], v);
}
int main(int argc, char** argv)
{
    const int W = atoi(argv[1]), M = atoi(argv[2]);
    std::vector<float> tab(W), u(M), out(M);
    for(int i = 0; i < W; i++) tab[i] = (float)i;
    // u spread over the texel range, including fine steps inside one texel
    for(int k = 0; k < M; k++) u[k] = (float)((0.5 + (double)k * (W - 1.0) / (M - 1.0)) / W);
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    cudaArray_t arr; cudaMallocArray(&arr, &ch, W, 1);
    cudaMemcpy2DToArray(arr, 0, 0, tab.data(), W * 4, W * 4, 1, cudaMemcpyHostToDevice);
    cudaResourceDesc rd = {}; rd.resType = cudaResourceTypeArray; rd.res.array.array = arr;
    cudaTextureDesc td = {}; td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear; td.readMode = cudaReadModeElementType; td.normalizedCoords = 1;
    cudaTextureObject_t t; cudaCreateTextureObject(&t, &rd, &td, nullptr);
    float *du, *dout; cudaMalloc(&du, M * 4); cudaMalloc(&dout, M * 4);
    cudaMemcpy(du, u.data(), M * 4, cudaMemcpyHostToDevice);
    k_fetch<<<(M + 255) / 256, 256>>>(t, du, dout, M, 0.5f);
    cudaError_t e = cudaDeviceSynchronize();
    if(e != cudaSuccess) { printf("error %s\n", cudaGetErrorString(e)); return 1; }
    cudaMemcpy(out.data(), dout, M * 4, cudaMemcpyDeviceToHost);
    FILE* f = fopen(argv[3], "wb"); fwrite(u.data(), 4, M, f); fwrite(out.data(), 4, M, f); fclose(f);
    printf("ok W=%d M=%d\n", W, M);
    return 0;
}
