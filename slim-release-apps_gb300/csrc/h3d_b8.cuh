// Batched BLOCK8 Kaczmarz double sweep over a table of problems (h3d_b8batch.cu).
//
// One launch per block parity covers every (problem, block, group of R right-hand sides) of
// the batch: problems may differ in grid size, PML, wavenumber (frequency) and mode, and each
// keeps its own stored row coefficients.  A CTA finds its problem by a binary search over the
// per-parity prefix counts of CTAs, copies the problem's descriptor into shared memory, and
// runs the block's 27 colours (54 for the middle parity) on its shared-memory boxes, the
// coefficient slab and inverse row norms of each colour arriving by one thread's bulk copy
// into an S-deep ring of buffers that complete on mbarriers.
#pragma once

#include <memory>
#include <vector>

#include "h3d_internal.cuh"
#include "h3d_vec.cuh"

namespace h3d {

// Device descriptor of one problem of a batched sweep.
template <typename T>
struct B8Prob {
    Op<T> op;
    const cplx<T> *coef;  // 12^3-block stored coefficients (store_block8_coefs layout)
    const T *rinv8;       // 1/||a_i||^2 in the same block- and colour-major order, 64 per slab
    long long col0;       // element offset of the problem's first column in x and b
    long long cstride;    // elements between two of its columns (its N)
    int c0;               // batch index of its first column (active flags)
    int nrhs;             // its columns
    int ngrp;             // groups of R columns (set per configuration)
    int adj;              // 1: rows of H^H
    int wnc;              // complex wavenumber (no real-coefficient interior blocks)
    int NI, NJ, NK;       // 12^3 blocks per axis
};

// Compiled (precision, R, S) configurations of the batched kernel.
struct B8Cfg {
    int r;    // right-hand sides per CTA
    int rpt;  // right-hand sides per thread (64 r / rpt threads)
    int s;    // depth of the coefficient ring
};
int b8_num_cfgs(bool fp64);
B8Cfg b8_cfg(bool fp64, int c);

template <typename T>
struct B8Batch {
    struct Item {
        Op<T> op;
        bool adj;
        long long col0;
        int c0, nrhs;
    };
    std::vector<Item> items;
    std::vector<std::unique_ptr<DevBuf>> coefs, rinvs;
    DevBuf desc, starts, errb;
    int cfg = -1;
    long long nctas[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int *err = nullptr;                       // device status: H3D_ERR_TIMEOUT after an expired wait
    unsigned long long wait_limit_ns = 1000000000ull;
    int verbose = 0;

    void add(const Op<T> &op, bool adj, long long col0, int c0, int nrhs) { items.push_back({op, adj, col0, c0, nrhs}); }
    // Device bytes setup() allocates: stored coefficients and block-ordered row norms.
    size_t bytes_needed() const;
    // Store every problem's coefficients and inverse row norms; clear the status word.
    int setup(cudaStream_t st);
    // Descriptor and CTA tables for configuration c (index into b8_cfg).
    int configure(int c, cudaStream_t st);
    // One forward + backward sweep on x (all columns of the batch) with right-hand side b
    // (null = 0); active: per-column flags (null = all); selftest: see the kernel.
    int dsweep(cplx<T> *x, const cplx<T> *b, T w, const int *active, cudaStream_t st, int selftest = 0);
    // Kernel launches of one double sweep (parities without blocks are skipped).
    int launches() const;
    // Time every configuration whose groups the columns fill on the scratch vector y (its
    // contents are overwritten) and keep the fastest; cached per batch shape.
    int tune(cplx<T> *y, long long len, cudaStream_t st);
    int max_nrhs() const;
};

}  // namespace h3d
