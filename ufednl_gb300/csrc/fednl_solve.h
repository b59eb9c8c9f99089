// fednl_solve.h -- the Option-B solve of one problem as plain device pointers, shared by the FP64
// and the mixed-precision translation units so that one cooperative launch can solve the systems
// of many live problems (the serving loop's batched solve).
#pragma once

#include <cuda_runtime.h>

#include <functional>

// elements of the FP64 cooperative solve's work array: the packed factor of the system augmented by
// the right-hand side as column d, then the current panel's unscaled rows (32 x (d + 1)) that the
// trailing update of the LDL^T factorization reads
inline size_t fednl_chol_work_elems(int d) { return (size_t)(d + 1) * (d + 2) / 2 + (size_t)32 * (d + 1); }

struct FednlSolveDesc {
    const double* H;       // packed upper FP64, d(d+1)/2
    int d;
    const double* lptr;    // device l (Option B), or nullptr to use lval (Option A: lambda)
    double lval;
    const double* g;       // device right-hand side
    double* dx;            // device solution
    double* xupd;          // device iterate (x -= dx) or nullptr
    double* work;          // fednl_chol_work_elems(d)
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

// The FP32 cooperative solve of the mixed-precision form (fednl_chol32c.cuh): its buffers, of
// fednl_solve32_bytes(d) device bytes in all, for d up to fednl_solve32_max_d().
struct FednlSolve32 {
    float* a;              // [ld][ld], ld = d rounded up to 32
    float* diag0;          // [d]
    float* linv;           // [ld][32]
    double* r;             // [d]
    double* acc;           // [d]
    float* accp;           // [2 d]
    const float* hh;       // H as FP32 pairs, packed upper column-major (hh, hl) and row-major
    const float* hl;       // (rh, rl): the FP32 load of the system and the float-float residual
    const float* rh;
    const float* rl;
    int* flag;             // [1]
    int refine;            // at most this many refinement steps after the first solve
    float tol;             // stop refining when the correction is at most tol of the solution
};
int fednl_solve32_max_d();
size_t fednl_solve32_bytes(int d);
// (H + l I) dx = g, x -= dx with the FP32 factor and FP64 refinement on `grid` CTAs (0: default);
// S.lptr is required.  An FP32 pivot that loses more than 18 bits hands the system to the FP64
// cooperative solve in the same launch (S.work, S.ybuf, S.rinv).
int fednl_device_optionb_solve32(const FednlSolveDesc& S, const FednlSolve32& E, cudaStream_t st, int grid);
int fednl_tune_chol32_grid(int d, const std::function<int(int)>& launch, cudaStream_t st, int* best_grid,
                           double* best_ms);

// fednl_mixed.cu: a mixed-precision handle's solve as a descriptor (and its stream)
struct fednl_mx_handle_s;
extern "C" int fednl_mx_solve_desc(struct fednl_mx_handle_s* h, FednlSolveDesc* desc, void** stream);
// 1 when the handle's solve is the FP32 shared-memory factor with refinement (fednl_chol32.cuh)
int fednl_mx_uses_chol32(struct fednl_mx_handle_s* h);
// those handles' solves in one launch, one CTA per system, on the given stream (host-synchronous)
int fednl_mx_solve32_batch(struct fednl_mx_handle_s* const* hs, int n, void* stream);
