// ensemble.hpp -- many mixed-form 2D Euler simulations of uneven sizes advanced
// together on one GPU.
//
// Every member is a full EulerSim (its own settings, maps, stack, initial condition,
// remaps, saves).  One ensemble iteration advances each active member by one of its own
// time steps.
//
// Single-launch iteration (the default where every member allows it, launch_ens_fused in
// csrc/ens_fused.cuh): precombination, advection, incompressibility check, the remap
// decision and the remaps (composition through the stack, fine-grid transforms, map push
// and reset), the psi solve (sample, rows, columns, inverse rows with the Lagrange
// combinations) and the coarse vorticity of every member run in one cooperative launch of
// persistent blocks that take tasks from per-wave device work queues.  Around it: one copy
// of the members' descriptors up, one memset of the launch's shared state and one copy of
// the members' E_inc and remap flags down, all captured in one CUDA graph once the shape is
// tuned.  The host then books each member's remap and does its particles and saves.  The
// autotuner tries every (resident blocks per SM, tiles per task) shape on the first
// iterations, round robin, and keeps the one with the lowest median iteration time.
//
// Two-phase iteration (the fallback): phase A (precombinations, advection, check) and phase
// B (sample, batched transforms per size class, spectral psi, psi nodes, coarse vorticity)
// in batched launches with the remaps one member at a time on the host between them; the
// persistent grid of each batched kernel is picked by timing the candidates on the first
// iteration, and each phase is a CUDA graph from the second on.
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
    // iteration form (set before init): 0 the two-phase iteration with the remaps on the host,
    // 1 the single launch, 2 (default) the autotuner's choice between the single launch in each of
    // its shapes and the two-phase iteration with the remaps in one batched launch
    int fused_mode = 2;
    long long wait_limit = 1ll << 24;   // polls before a grid barrier of a batched launch gives up
    bool fused_available() const { return fused_ok_; }
    bool fused() const { return fused_ok_ && fused_minb != 0; }   // the form in use is the single launch
    std::string fused_why;           // why the single-launch iteration is unavailable
    int fused_minb = 0, fused_blocks = 0, fused_g = 0, last_waves = 0;
    // register budget (blocks per SM; 0: the two-phase iteration with batched remaps), grid, tiles
    // per task, median wall time of an iteration
    struct Shape { int minb, blocks, g; double ms; };
    std::vector<Shape> tuning;       // the autotuner's table
    void set_wait_limit(long long polls);
    // profiling counters of the single launch (kProfValues: cycles and tasks per stage, barrier
    // cycles, nanoseconds per wave), summed over the iterations since profiling was switched on
    int set_profiling(bool on);
    int read_profile(unsigned long long* out);
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
        // the single-launch iteration: fine-grid transforms and per-member work arrays
        fft::Plan2D pf;
        float* freal = nullptr;
        float2* fw1 = nullptr;
        float2* fw2 = nullptr;
        long long freal_stride = 0, fw1_stride = 0, fw2_stride = 0;
    };
    int phase_a();
    int phase_b();
    int launch(int kind, int blocks_now);
    int tune(const std::vector<int>& kinds);
    int capture(int which, cudaGraphExec_t* exec);
    void drop_graphs();
    int check(cudaError_t e, const char* what);
    int init_fused();
    int step_fused(const Shape& sh);
    int step_two_phase(bool batched_remaps);
    int fused_sequence(const Shape& sh);   // descriptors up, state zeroed, the launch, results down
    int remap_launch();                     // the two-phase iteration's batched remaps (h_rem_)

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
    // single-launch iteration
    bool fused_ok_ = false, broken_ = false, fused_tuned_ = false, remap_pending_ = false;
    EnsMember* h_rem_ = nullptr;             // remap descriptors of the two-phase iteration (pinned)
    EnsMember* d_rem_ = nullptr;
    EnsClass* d_cls_ = nullptr;
    unsigned char* d_fsh_ = nullptr;         // EnsShared, then M E_inc (FP64 bits), then M remap flags
    unsigned char* h_fsh_ = nullptr;         // pinned copy
    size_t fsh_bytes_ = 0;
    int tab_values_ = 0, work_values_ = 0, sms_ = 0;
    std::vector<Shape> cands_;
    std::vector<std::vector<float>> samples_;
    int tune_iter_ = 0;
    cudaGraphExec_t fgraph_ = nullptr;
    unsigned long long* d_prof_ = nullptr;   // profiling counters (null: off)
};

}  // namespace cmm
