// The rescue model's float log (gi_model.h) over doubles read from argv[1], floats written to
// argv[2] (the test compares them with the host's log).
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "gi_model.h"

__global__ void k_log(const double* in, float* out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = model_log(in[i]);
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    std::vector<double> x;
    double v;
    while (fread(&v, sizeof v, 1, f) == 1) x.push_back(v);
    fclose(f);
    const size_t n = x.size();
    double* d_in = nullptr;
    float* d_out = nullptr;
    if (cudaMalloc(&d_in, n * sizeof(double) + 8) != cudaSuccess || cudaMalloc(&d_out, n * sizeof(float) + 4) != cudaSuccess)
        return 3;
    cudaMemcpy(d_in, x.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    k_log<<<1024, 256>>>(d_in, d_out, n);
    std::vector<float> y(n);
    if (cudaMemcpy(y.data(), d_out, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    FILE* g = fopen(argv[2], "wb");
    if (!g) return 2;
    fwrite(y.data(), sizeof(float), n, g);
    fclose(g);
    return 0;
}
