// ensemble.hpp -- many mixed-form 2D Euler simulations of uneven sizes advanced
// together on one GPU.
//
// Every member is a full EulerSim (its own settings, maps, stack, initial condition,
// remaps, saves).  One ensemble iteration advances each active member by one of its own
// time steps; the per-step work of all members runs in a handful of launches:
//   phase A: descriptors up, precombinations, map advection, incompressibility check,
//            the members' E_inc down (one 8-byte value each, one copy);
//   host:    remaps of the members whose E_inc asks for one, psi rotation;
//   phase B: descriptors up, omega on the vort grids, one batched R2C per size class, the
//            spectral psi, one batched C2R (4 planes) per size class, psi nodes and Lagrange
//            combinations, coarse vorticity.
// Members of one size class share contiguous FFT buffers, so each class transforms in one
// batched transform (csrc/fft.hpp).  The batched kernels walk a work list of 256-thread tiles with a
// persistent grid whose size per kernel is picked by timing the candidates on the first
// iteration (every batched kernel is idempotent within a step, so the trials cost time but
// change nothing).  From the second iteration on each phase is a CUDA graph, re-captured
// when a size class finishes.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "mixed.hpp"
#include "sim.hpp"

namespace cmm {

class EnsembleSim {
public:
    explicit EnsembleSim(const std::vector<Settings>& members);
    ~EnsembleSim();

    int set_initial_discrete(int i, const double* host, size_t n);
    int init();          // every member's init, then the ensemble's buffers, plans and work lists
    int step();          // one iteration: 0, 1 (every member done) or an error
    int run();           // iterate until every member is done, then finish each member
    bool done() const;

    int size() const { return (int)m_.size(); }
    EulerSim& member(int i) { return *m_[(size_t)i]; }

    std::string err;
    cudaStream_t stream = nullptr;
    bool use_graphs = true;
    long long member_steps = 0;      // member time steps taken
    long long iterations = 0;
    long long launches = 0;          // batched launches + transform kernels + per-member remap work
    int blocks[kEnsKinds] = {0};     // tuned persistent grid per kernel kind
    int tiles[kEnsKinds] = {0};      // work-list length per kernel kind

private:
    struct SizeClass {
        int nv = 0, np = 0;              // vort and psi grid sizes
        std::vector<int> members;
        float* real = nullptr;           // per member max(Nv, 4 Np) floats
        float2* spec = nullptr;          // per member Nv_fft
        float2* spec4 = nullptr;         // per member 4 Np_fft
        long long real_stride = 0, spec_stride = 0, spec4_stride = 0;
        fft::Plan2D pv, pp;             // FP32 transforms of the vort and psi grids
        bool active = true;
    };
    int phase_a();
    int phase_b();
    int launch(int kind, int blocks_now);
    int tune(const std::vector<int>& kinds);
    int capture(int which, cudaGraphExec_t* exec);
    void drop_graphs();
    int check(cudaError_t e, const char* what);

    std::vector<std::unique_ptr<EulerSim>> m_;
    std::vector<SizeClass> cls_;
    // descriptors, pinned and on the device, one pair per phase: phase A's are written by
    // the host only after the previous phase A has completed (the E_inc read synchronises),
    // phase B's only after the next phase A, which follows the previous phase B in the stream
    EnsMember* h_mem_[2] = {nullptr, nullptr};
    EnsMember* d_mem_[2] = {nullptr, nullptr};
    int* d_cum_[kEnsKinds] = {nullptr};      // work lists
    unsigned long long* d_einc_ = nullptr;
    double* h_einc_ = nullptr;               // pinned
    int lpn_log2_ = 3;
    int ti_ = 30;
    bool initialised_ = false, tuned_ = false, own_stream_ = false;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};
    std::vector<int> stepping_;              // members that took this iteration's step
};

}  // namespace cmm
