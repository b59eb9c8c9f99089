// fednl_solve.h -- the Option-B solve of one problem as plain device pointers, shared by the FP64
// and the mixed-precision translation units so that one cooperative launch can solve the systems
// of many live problems (the serving loop's batched solve).
#pragma once

#include <cuda_runtime.h>

#include <functional>

struct FednlSolveDesc {
    const double* H;       // packed upper FP64, d(d+1)/2
    int d;
    const double* lptr;    // device l (Option B), or nullptr to use lval (Option A: lambda)
    double lval;
    const double* g;       // device right-hand side
    double* dx;            // device solution
    double* xupd;          // device iterate (x -= dx) or nullptr
    double* work;          // (d+1)(d+2)/2
    double* ybuf;          // d
    double* rinv;          // d
    unsigned* bar;         // 4 x u32
    int* status;
    double* stats;         // stats[0] = ||g|| with record
    double* hist;
    double* ls;            // line-search state or nullptr
    int* round_ctr;
    int hist_cap;
    int record;
};

// fednl_gpu.cu
int fednl_solve_batch_launch(const FednlSolveDesc* descs, int n, void* stream);
// the cooperative Cholesky's CTA count for dimension d, measured with launch(G) on the caller's
// stream and cached per d for the process
int fednl_tune_chol_grid(int d, const std::function<int(int)>& launch, cudaStream_t st, int* best_grid,
                         double* best_ms);

// fednl_mixed.cu: a mixed-precision handle's solve as a descriptor (and its stream)
struct fednl_mx_handle_s;
extern "C" int fednl_mx_solve_desc(struct fednl_mx_handle_s* h, FednlSolveDesc* desc, void** stream);
// 1 when the handle's solve is the FP32 shared-memory factor with refinement (fednl_chol32.cuh)
int fednl_mx_uses_chol32(struct fednl_mx_handle_s* h);
// those handles' solves in one launch, one CTA per system, on the given stream (host-synchronous)
int fednl_mx_solve32_batch(struct fednl_mx_handle_s* const* hs, int n, void* stream);
