/*
 * siminf_reduce.cu -- the consumers of a trajectory on the device: the
 * long-format extraction of SimInf_trajectory and the three prevalence
 * levels of prevalence(), reading U (or V) where the solver left it in HBM,
 * so that a caller that wants a few series out of a 5.8 GB trajectory copies
 * those series, not the trajectory.
 *
 * Trajectory (src/misc/SimInf_trajectory.c:566-620, SimInf_u_dense2df and
 * SimInf_v_dense2df): for each requested compartment (or continuous state
 * variable) one column of length ncol * n_id, row (col, l) = the value of
 * node id[l] in column col of U, columns in U's order (replicate-major, then
 * time), nodes in the order given.
 *
 * Prevalence (R/prevalence.R:72-96, calculate_prevalence): per node and
 * column, cases = the sum of the case compartments and population = the
 * sum of the population compartments, both set to zero where the condition
 * is false; then level 1: sum(cases) / sum(population) over the nodes;
 * level 2: #(cases > 0) / #(population > 0); level 3: cases / population
 * per node.  Sums are exact in 64-bit integers and each quotient is one IEEE
 * division, so the results equal the reference's bit for bit.
 *
 * The condition is a program in postfix form (siminf_gpu_prevalence_spec),
 * checked on the host before a launch so that its evaluation stays inside
 * a fixed stack.
 *
 * Both kernels read each node's block of a column once and are bound by
 * HBM bandwidth: bytes read = ncol * n_id * stride * element size.
 */
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_capi_internal.h"
#include "siminf_plan.h"

using namespace siminf;

namespace {

/* A block of REDUCE_BLOCK threads takes NODES_PER_BLOCK nodes of one
 * column, NODES_PER_BLOCK / REDUCE_BLOCK per thread: few enough blocks that
 * the per-block atomics of levels 1 and 2 stay off the critical path, and
 * several loads in flight per thread. */
enum { REDUCE_BLOCK = 256, NODES_PER_BLOCK = 8192, COND_STACK = 16, COND_MAX_OPS = 256 };

/* The condition of one node in one column: the postfix program over the
 * node's compartments u[0 .. Nc). */
__device__ long long eval_condition(const int2 *prog, int n, const int *u)
{
    long long st[COND_STACK];
    int sp = 0;
    for (int k = 0; k < n; k++) {
        const int op = prog[k].x, arg = prog[k].y;
        switch (op) {
        case SIMINF_GPU_COND_COMPARTMENT:
            st[sp++] = u[arg];
            break;
        case SIMINF_GPU_COND_CONST:
            st[sp++] = arg;
            break;
        case SIMINF_GPU_COND_NEG:
            st[sp - 1] = -st[sp - 1];
            break;
        case SIMINF_GPU_COND_NOT:
            st[sp - 1] = st[sp - 1] == 0;
            break;
        default: {
            const long long b = st[--sp], a = st[sp - 1];
            long long r = 0;
            switch (op) {
            case SIMINF_GPU_COND_ADD: r = a + b; break;
            case SIMINF_GPU_COND_SUB: r = a - b; break;
            case SIMINF_GPU_COND_MUL: r = a * b; break;
            case SIMINF_GPU_COND_EQ: r = a == b; break;
            case SIMINF_GPU_COND_NE: r = a != b; break;
            case SIMINF_GPU_COND_LT: r = a < b; break;
            case SIMINF_GPU_COND_LE: r = a <= b; break;
            case SIMINF_GPU_COND_GT: r = a > b; break;
            case SIMINF_GPU_COND_GE: r = a >= b; break;
            case SIMINF_GPU_COND_AND: r = (a != 0) & (b != 0); break;
            case SIMINF_GPU_COND_OR: r = (a != 0) | (b != 0); break;
            }
            st[sp - 1] = r;
        }
        }
    }
    return st[0];
}

/* Sum of a long long over the block; the total is valid in thread 0. */
__device__ __forceinline__ long long block_sum(long long x, long long *sh)
{
    for (int o = 16; o > 0; o >>= 1)
        x += __shfl_down_sync(0xFFFFFFFFu, x, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0)
        sh[w] = x;
    __syncthreads();
    long long t = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < REDUCE_BLOCK / 32; k++)
            t += sh[k];
    return t;
}

struct PrevArgs {
    const int *U;
    long long Nn, ncol, n_id;
    int Nc;
    const int *id;          /* zero-based nodes, or nullptr for all */
    uint32_t cases, pop;
    int level;
    const int2 *cond;
    int ncond;
    unsigned long long *acc;    /* levels 1 and 2: [block][2] partial sums */
    double *out;                /* level 3: [ncol][n_id] */
};

/* The Nc values of a node's block u, with one 16-byte load when Nc is 4
 * (NCV = 4; a node's block then starts at a multiple of 16 bytes). */
template <int NCV>
__device__ __forceinline__ void node_counts(const int *u, int Nc, uint32_t cases, uint32_t pop,
                                            long long &num, long long &den)
{
    if constexpr (NCV == 4) {
        const int4 w = *reinterpret_cast<const int4 *>(u);
        const int v[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            num += ((cases >> c) & 1u) ? v[c] : 0;
            den += ((pop >> c) & 1u) ? v[c] : 0;
        }
    } else {
        for (int c = 0; c < Nc; c++) {
            const int v = u[c];
            num += ((cases >> c) & 1u) ? v : 0;
            den += ((pop >> c) & 1u) ? v : 0;
        }
    }
}

/* One block: NODES_PER_BLOCK nodes of one column. */
template <int NCV>
__global__ void __launch_bounds__(REDUCE_BLOCK) k_prevalence(PrevArgs a)
{
    __shared__ long long sh[REDUCE_BLOCK / 32];
    const long long chunks = (a.n_id + NODES_PER_BLOCK - 1) / NODES_PER_BLOCK;
    const long long col = blockIdx.x / chunks;
    const long long base = (blockIdx.x % chunks) * NODES_PER_BLOCK;
    long long tnum = 0, tden = 0;
#pragma unroll 8
    for (int k = 0; k < NODES_PER_BLOCK / REDUCE_BLOCK; k++) {
        const long long l = base + k * REDUCE_BLOCK + threadIdx.x;
        if (l >= a.n_id)
            break;
        const long long node = a.id ? a.id[l] : l;
        const int *u = a.U + (col * a.Nn + node) * a.Nc;
        long long num = 0, den = 0;
        node_counts<NCV>(u, a.Nc, a.cases, a.pop, num, den);
        if (a.ncond && !eval_condition(a.cond, a.ncond, u))
            num = den = 0;
        if (a.level == 3) {
            a.out[col * a.n_id + l] = (double) num / (double) den;
        } else if (a.level == 2) {
            tnum += num > 0;
            tden += den > 0;
        } else {
            tnum += num;
            tden += den;
        }
    }
    if (a.level != 3) {
        /* the block's partial sums, summed per column by k_prevalence_final
         * in block order */
        tnum = block_sum(tnum, sh);
        tden = block_sum(tden, sh);
        if (threadIdx.x == 0) {
            a.acc[2 * blockIdx.x] = (unsigned long long) tnum;
            a.acc[2 * blockIdx.x + 1] = (unsigned long long) tden;
        }
    }
}

/* Per column, the sums of its blocks' partial sums (chunks blocks per
 * column, column-major in the grid), then the quotient. */
__global__ void k_prevalence_final(const unsigned long long *acc, long long ncol,
                                   long long chunks, double *out)
{
    const long long col = blockIdx.x * (long long) blockDim.x + threadIdx.x;
    if (col >= ncol)
        return;
    unsigned long long num = 0, den = 0;
    for (long long c = 0; c < chunks; c++) {
        num += acc[2 * (col * chunks + c)];
        den += acc[2 * (col * chunks + c) + 1];
    }
    out[col] = (double) (long long) num / (double) (long long) den;
}

/* One block: NODES_PER_BLOCK nodes of one column; T is int (U) or double
 * (V); VEC4: int U with stride 4, one 16-byte load per node. */
template <class T, bool VEC4>
__global__ void __launch_bounds__(REDUCE_BLOCK) k_trajectory(const T *M, long long Nn, int stride,
                                                             long long ncol, const int *id,
                                                             long long n_id, const int *var,
                                                             int n_var, T *out)
{
    const long long chunks = (n_id + NODES_PER_BLOCK - 1) / NODES_PER_BLOCK;
    const long long col = blockIdx.x / chunks;
    const long long base = (blockIdx.x % chunks) * NODES_PER_BLOCK;
    const size_t plane = (size_t) ncol * n_id;
#pragma unroll 4
    for (int k = 0; k < NODES_PER_BLOCK / REDUCE_BLOCK; k++) {
        const long long l = base + k * REDUCE_BLOCK + threadIdx.x;
        if (l >= n_id)
            break;
        const long long node = id ? id[l] : l;
        const T *m = M + (col * Nn + node) * stride;
        if constexpr (VEC4) {
            const int4 w = *reinterpret_cast<const int4 *>(m);
            const int v[4] = {w.x, w.y, w.z, w.w};
            for (int i = 0; i < n_var; i++) {
                const int c = var[i];
                out[i * plane + col * n_id + l] = c == 0 ? v[0] : c == 1 ? v[1] : c == 2 ? v[2] : v[3];
            }
        } else {
            for (int i = 0; i < n_var; i++)
                out[i * plane + col * n_id + l] = m[var[i]];
        }
    }
}

int fail(int code, const char *msg)
{
    capi_set_status(code, -1, -1, -1, 0, 0, msg);
    return code;
}

/* Device copy of the zero-based node list (one-based ids in), checked. */
int upload_ids(const int *id, int n_id, int Nn, int **d_id, cudaStream_t st)
{
    *d_id = nullptr;
    if (!id)
        return 0;
    std::vector<int> z((size_t) n_id);
    for (int i = 0; i < n_id; i++) {
        if (id[i] < 1 || id[i] > Nn)
            return fail(SIMINF_GPU_ERR_NODE_OUT_OF_BOUNDS, "node index out of range");
        z[i] = id[i] - 1;
    }
    cudaError_t e = cudaMallocAsync((void **) d_id, z.size() * sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(*d_id, z.data(), z.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);      /* z leaves scope */
    return e == cudaSuccess ? 0 : capi_cuda_fail(e, "node index upload");
}

/* A condition the kernel can evaluate: every operator finds its operands,
 * the stack stays within COND_STACK, one value remains, compartments are
 * in range, and the last operator gives TRUE or FALSE. */
int check_condition(const int *prog, int n, int Nc)
{
    if (n < 0 || n > COND_MAX_OPS)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "condition too long");
    if (n == 0)
        return 0;
    int sp = 0, refs = 0;
    for (int k = 0; k < n; k++) {
        const int op = prog[2 * k], arg = prog[2 * k + 1];
        int need, push;
        switch (op) {
        case SIMINF_GPU_COND_COMPARTMENT:
            if (arg < 0 || arg >= Nc)
                return fail(SIMINF_GPU_ERR_INVALID_MODEL, "condition: compartment out of range");
            refs++;
            need = 0, push = 1;
            break;
        case SIMINF_GPU_COND_CONST: need = 0, push = 1; break;
        case SIMINF_GPU_COND_NEG:
        case SIMINF_GPU_COND_NOT: need = 1, push = 1; break;
        case SIMINF_GPU_COND_ADD: case SIMINF_GPU_COND_SUB: case SIMINF_GPU_COND_MUL:
        case SIMINF_GPU_COND_EQ: case SIMINF_GPU_COND_NE: case SIMINF_GPU_COND_LT:
        case SIMINF_GPU_COND_LE: case SIMINF_GPU_COND_GT: case SIMINF_GPU_COND_GE:
        case SIMINF_GPU_COND_AND: case SIMINF_GPU_COND_OR: need = 2, push = 1; break;
        default:
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "condition: unknown operator");
        }
        if (sp < need)
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "condition: missing operand");
        sp = sp - need + push;
        if (sp > COND_STACK)
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "condition: too deeply nested");
    }
    const int last = prog[2 * (n - 1)];
    const bool logical = last == SIMINF_GPU_COND_NOT ||
                         (last >= SIMINF_GPU_COND_EQ && last <= SIMINF_GPU_COND_OR);
    if (sp != 1 || !logical || refs == 0)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL,
                    "The condition must be either 'TRUE' or 'FALSE' for every node and time step.");
    return 0;
}

long long grid_of(long long ncol, long long n_id)
{
    return ncol * ((n_id + NODES_PER_BLOCK - 1) / NODES_PER_BLOCK);
}

template <class T>
int trajectory_impl(const T *d_M, int Nn, int stride, int ncol, const int *var, int n_var,
                    const int *id, int n_id, T *out, cudaStream_t st,
                    siminf_gpu_reduce_stats *rs)
{
    capi_clear_status();
    if (!d_M || !out || !var || Nn < 1 || stride < 1 || ncol < 1 || n_var < 1 ||
        (id && n_id < 1))
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "invalid trajectory arguments");
    for (int i = 0; i < n_var; i++)
        if (var[i] < 1 || var[i] > stride)
            return fail(SIMINF_GPU_ERR_INVALID_MODEL, "compartment index out of range");
    const long long nid = id ? n_id : Nn;
    const long long blocks = grid_of(ncol, nid);
    if (blocks > INT_MAX)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "trajectory too large for one launch");
    int *d_id = nullptr, *d_var = nullptr;
    T *d_out = nullptr;
    int rc = upload_ids(id, n_id, Nn, &d_id, st);
    if (rc)
        return rc;
    std::vector<int> zv((size_t) n_var);
    for (int i = 0; i < n_var; i++)
        zv[i] = var[i] - 1;
    const size_t out_n = (size_t) n_var * ncol * nid;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaMallocAsync((void **) &d_var, zv.size() * sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_var, zv.data(), zv.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMallocAsync((void **) &d_out, out_n * sizeof(T), st);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        cudaEventRecord(e0, st);
        if (std::is_same<T, int>::value && stride == 4 && ((uintptr_t) d_M & 15) == 0)
            k_trajectory<T, true><<<(unsigned) blocks, REDUCE_BLOCK, 0, st>>>(
                d_M, Nn, stride, ncol, d_id, nid, d_var, n_var, d_out);
        else
            k_trajectory<T, false><<<(unsigned) blocks, REDUCE_BLOCK, 0, st>>>(
                d_M, Nn, stride, ncol, d_id, nid, d_var, n_var, d_out);
        e = cudaGetLastError();
        cudaEventRecord(e1, st);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, out_n * sizeof(T), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    float ms = 0;
    if (e == cudaSuccess && rs) {
        cudaEventElapsedTime(&ms, e0, e1);
        rs->ms_kernel = ms;
        rs->ms_total = std::chrono::duration<double, std::milli>(
                           std::chrono::steady_clock::now() - t0).count();
        rs->bytes_read = (long long) ncol * nid * stride * (long long) sizeof(T);
        rs->bytes_written = (long long) (out_n * sizeof(T));
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFreeAsync(d_out, st);
    cudaFreeAsync(d_var, st);
    if (d_id)
        cudaFreeAsync(d_id, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = e2;
    return e == cudaSuccess ? 0 : capi_cuda_fail(e, "trajectory");
}

}  // namespace

extern "C" {

int siminf_gpu_trajectory_u(const int *d_U, int Nn, int Nc, int ncol, const int *compartments,
                            int n_compartments, const int *id, int n_id, int *out,
                            void *cuda_stream, siminf_gpu_reduce_stats *stats)
{
    return trajectory_impl<int>(d_U, Nn, Nc, ncol, compartments, n_compartments, id, n_id, out,
                                (cudaStream_t) cuda_stream, stats);
}

int siminf_gpu_trajectory_v(const double *d_V, int Nn, int Nd, int ncol, const int *variables,
                            int n_variables, const int *id, int n_id, double *out,
                            void *cuda_stream, siminf_gpu_reduce_stats *stats)
{
    return trajectory_impl<double>(d_V, Nn, Nd, ncol, variables, n_variables, id, n_id, out,
                                   (cudaStream_t) cuda_stream, stats);
}

int siminf_gpu_prevalence(const int *d_U, int Nn, int Nc, int ncol,
                          const siminf_gpu_prevalence_spec *spec, const int *id, int n_id,
                          double *out, void *cuda_stream, siminf_gpu_reduce_stats *stats)
{
    capi_clear_status();
    const cudaStream_t st = (cudaStream_t) cuda_stream;
    if (!d_U || !spec || !out || Nn < 1 || Nc < 1 || Nc > 32 || ncol < 1 || (id && n_id < 1))
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "invalid prevalence arguments");
    if (spec->level < 1 || spec->level > 3)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL,
                    "'level' must be an integer with a value 1, 2 or 3.");
    const uint32_t all = Nc == 32 ? 0xFFFFFFFFu : ((1u << Nc) - 1u);
    if (!spec->cases || !spec->population || (spec->cases & ~all) || (spec->population & ~all))
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "Invalid 'formula' specification.");
    int rc = check_condition(spec->condition, spec->n_condition, Nc);
    if (rc)
        return rc;
    const long long nid = id ? n_id : Nn;
    const long long blocks = grid_of(ncol, nid);
    if (blocks > INT_MAX)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL, "prevalence too large for one launch");
    int *d_id = nullptr;
    if ((rc = upload_ids(id, n_id, Nn, &d_id, st)))
        return rc;
    const size_t out_n = spec->level == 3 ? (size_t) ncol * nid : (size_t) ncol;
    int2 *d_cond = nullptr;
    unsigned long long *d_acc = nullptr;
    double *d_out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaMallocAsync((void **) &d_out, out_n * sizeof(double), st);
    if (e == cudaSuccess && spec->n_condition > 0) {
        e = cudaMallocAsync((void **) &d_cond, (size_t) spec->n_condition * sizeof(int2), st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_cond, spec->condition,
                                (size_t) spec->n_condition * sizeof(int2),
                                cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess && spec->level != 3)
        e = cudaMallocAsync((void **) &d_acc, (size_t) 2 * blocks * sizeof(unsigned long long), st);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        PrevArgs a;
        a.U = d_U;
        a.Nn = Nn;
        a.ncol = ncol;
        a.n_id = nid;
        a.Nc = Nc;
        a.id = d_id;
        a.cases = spec->cases;
        a.pop = spec->population;
        a.level = spec->level;
        a.cond = d_cond;
        a.ncond = spec->n_condition;
        a.acc = d_acc;
        a.out = d_out;
        cudaEventRecord(e0, st);
        if (Nc == 4 && ((uintptr_t) d_U & 15) == 0)
            k_prevalence<4><<<(unsigned) blocks, REDUCE_BLOCK, 0, st>>>(a);
        else
            k_prevalence<0><<<(unsigned) blocks, REDUCE_BLOCK, 0, st>>>(a);
        e = cudaGetLastError();
        if (e == cudaSuccess && spec->level != 3) {
            k_prevalence_final<<<(unsigned) ((ncol + 255) / 256), 256, 0, st>>>(
                d_acc, ncol, (nid + NODES_PER_BLOCK - 1) / NODES_PER_BLOCK, d_out);
            e = cudaGetLastError();
        }
        cudaEventRecord(e1, st);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, out_n * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        stats->ms_kernel = ms;
        stats->ms_total = std::chrono::duration<double, std::milli>(
                              std::chrono::steady_clock::now() - t0).count();
        stats->bytes_read = (long long) ncol * nid * Nc * (long long) sizeof(int);
        stats->bytes_written = (long long) (out_n * sizeof(double));
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFreeAsync(d_out, st);
    if (d_cond)
        cudaFreeAsync(d_cond, st);
    if (d_acc)
        cudaFreeAsync(d_acc, st);
    if (d_id)
        cudaFreeAsync(d_id, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        e = e2;
    return e == cudaSuccess ? 0 : capi_cuda_fail(e, "prevalence");
}

int siminf_gpu_plan_outputs(const siminf_gpu_plan *p, const int **d_U, const double **d_V,
                            int *ncol)
{
    if (!p || !p->ran)
        return fail(SIMINF_GPU_ERR_INVALID_MODEL,
                    "Please run the model first, the trajectory is empty.");
    if (d_U)
        *d_U = p->s.U;
    if (d_V)
        *d_V = p->s.V;
    if (ncol)
        *ncol = p->s.Nrep * p->s.tlen;
    return 0;
}

}  /* extern "C" */
