// Host orchestration of the design-matrix path on one GPU: device copies of the
// model tables, device-resident frame batches, and the launch sequence
//   ghosts -> neighbour lists -> clusters -> owner / type buckets -> A rows.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "dev.cuh"
#include "model.h"

namespace cg {

void cuda_check(cudaError_t e, const char* what);

// Model tables uploaded to the device (immutable after creation).
struct DeviceModel {
    cgd::ModelDev dev{};
    std::vector<void*> allocs;
    int max_allowed3 = 0, max_allowed4 = 0;
    explicit DeviceModel(const Model& m, int vir_pchunk);
    ~DeviceModel();
    DeviceModel(const DeviceModel&) = delete;
    DeviceModel& operator=(const DeviceModel&) = delete;
};

// Host-side flattened frames (one A-matrix row block per frame).
struct FrameBatch {
    int nframes = 0, first_index = 0;
    std::vector<int> natoms, stress_rows, energy_rows;
    std::vector<int64_t> atom_ofs, ghost_ofs, row_ofs;
    std::vector<cgd::BoxDev> box;
    std::vector<int> type;
    std::vector<double> xyz;
    std::vector<double> b;        // labels in A row order (src/A_Matrix.C:294-553)
    int64_t nrows = 0, natoms_total = 0, nghosts = 0;
};

FrameBatch make_batch(const Model& m, const std::vector<Frame>& frames, int first_index);

// The same batch resident in device memory.
struct DeviceFrames {
    cgd::FramesDev dev{};
    int nframes = 0;
    int64_t nrows = 0, natoms_total = 0, nghosts = 0;
    std::vector<int64_t> atom_ofs_host, row_ofs_host;
    std::vector<int> natoms_host;
    std::vector<void*> allocs;
    ~DeviceFrames();
};

struct AssembleStats {
    int64_t pairs2 = 0, list3 = 0, list4 = 0, triplets = 0, quads = 0;
    int64_t power_evals3 = 0, power_evals4 = 0;   // sum over clusters of n_allowed
};

class Session {
   public:
    Session(const Model& m, int device);
    ~Session();
    const Model& model() const { return model_; }
    cudaStream_t stream() const { return stream_; }
    std::unique_ptr<DeviceFrames> upload(const FrameBatch& fb);
    // A (device pointer, row-major, lda >= tot_all) receives the batch's rows.
    void assemble(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats);

   private:
    Model model_;
    int device_;
    cudaStream_t stream_ = nullptr;
    std::unique_ptr<DeviceModel> dm_;
};

}  // namespace cg
