// Learned preconditioner: parameters, checkpoint and trainer (learned.cu), and
// the flexible CG that applies it (flexcg.cu).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace prgpu {

struct Ctx;

// fp32 parameter vector: W1 [64 out][64 in], b1, W2 [64][64], b2, w3 [64], b3
constexpr int P_W1 = 0, P_B1 = 4096, P_W2 = 4160, P_B2 = 8256, P_W3 = 8320, P_B3 = 8384, P_COUNT = 8385;
constexpr int FEAT_USED = 55;            // features 55..63 are zero
constexpr float TARGET_CLIP = 64.f;      // |training target| bound
constexpr uint32_t CKPT_VERSION = 1;

struct MlpWeights {          // device pointers
    const __nv_bfloat16* w1; // [64][64]
    const __nv_bfloat16* w2;
    const float* p;          // fp32 parameters
};

void write_checkpoint(const char* path, const float* hp, const float* hm, const float* hv, i64 step, uint64_t seed,
                      i64 epoch);
void read_checkpoint(const char* path, std::vector<float>& hp, std::vector<float>& hm, std::vector<float>& hv,
                     i64& step, uint64_t& seed, i64& epoch);
void init_params(std::vector<float>& p, uint64_t seed);

// Owns the network's parameters, Adam state and the training samples on one device.
struct Trainer {
    int device = 0;
    uint64_t seed = 0;
    cudaStream_t stream = nullptr;
    float *p = nullptr, *g = nullptr, *mo = nullptr, *ve = nullptr;   // P_COUNT each
    __nv_bfloat16 *w1b = nullptr, *w2b = nullptr;                     // bf16 mirrors
    double* loss = nullptr;
    int* err = nullptr;
    __nv_bfloat16* feat = nullptr;   // [cap][64]
    float* target = nullptr;         // [cap]
    int* order = nullptr;            // current epoch's sample order
    i64 nsamples = 0, cap = 0, cursor = 0, step = 0, epoch = 0, record_calls = 0;

    Trainer(int device, uint64_t seed);
    ~Trainer();
    void set_params(const float* hp, const float* hm, const float* hv);
    void reserve(i64 want);
    MlpWeights weights() const;
    i64 record(Ctx& c, int rows_per_depth);
    double train(int steps, int batch, float lr);
    double gradients(const __nv_bfloat16* dfeat, const float* dtarget, i64 n, float* hgrad);
    void forward(const __nv_bfloat16* dfeat, i64 n, float* dy);
    void save(const char* path);
    void load(const char* path);
};

}  // namespace prgpu
