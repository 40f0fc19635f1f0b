/*
 * siminf_schedule.h -- the device event planner (siminf_schedule.cu): the
 * scheduled events of a chunk of days classified, checked and split into
 * the wavefronts and per-node lists the solver kernels read, on the GPU.
 */
#ifndef SIMINF_SCHEDULE_H
#define SIMINF_SCHEDULE_H

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/siminf_gb300.h"
#include "siminf_plan.h"

namespace siminf {

/* The columns of a chunk's events in device staging buffers (index 0 is
 * the chunk's first event). */
struct SchedCols {
    const int *time, *event, *node, *dest, *n, *select, *shift;
    const double *proportion;
};

/* A planned failure found on the device (the fields of PlannedErr). */
struct SchedPlanned {
    int day, code, index, node, phase;
};

/* What the planner's kernels report across chunks. */
struct SchedStatus {
    unsigned long long bad;     /* first event out of (time, E1 before E2) order, or ~0 */
    int max_select, max_shift;
    unsigned n_planned;
    SchedPlanned planned[1];    /* MAX_PLANNED entries follow */
};

/* One planned chunk, as the host needs it to launch the chunk's days. */
struct SchedChunk {
    long long n1 = 0, n2 = 0;               /* E1 events, external transfers */
    unsigned long long bad = ~0ULL;         /* the status after this chunk: first */
    int max_select = 0, max_shift = 0;      /* event out of order, select / shift maxima */
    std::vector<long long> off;             /* nd + 1: first transfer of each day */
    std::vector<std::vector<long long>> waves;  /* per day: wave sizes */
    std::vector<int> deep;                  /* days left to the host planner */
};

class DevScheduler {
public:
    enum { MAX_CHUNK_DAYS = 16, MAX_ROUNDS = 2048, MAX_PLANNED = 65536 };

    ~DevScheduler();
    /* Buffers for chunks of at most max_events events; Nn nodes; nsel the
     * number of select columns events may use (INT_MAX: no bound). */
    cudaError_t init(long long max_events, int Nn, int nsel, cudaStream_t st);

    /* Staging buffers the caller fills with a chunk's columns before
     * plan_chunk (capacity: max_events). */
    int *time = nullptr, *event = nullptr, *node = nullptr, *dest = nullptr, *n = nullptr,
        *select = nullptr, *shift = nullptr;
    double *proportion = nullptr;

    /* Plan events [lo, lo + m), days d0 .. d0 + nd - 1, day j holding
     * events [lo + bounds[j], lo + bounds[j + 1]) (bounds[nd] = m).  The
     * predecessor of event lo (for the order check) is (prev_time,
     * prev_event) if has_prev.  Writes the chunk's transfers in wave order
     * to e2_out (n2 records), its E1 records by node to e1_out with the
     * per-node offsets e1_ptr (Nn + 1 entries), and, if wave_out is not
     * null, each transfer's zero-based wave to wave_out[event index].  The
     * host reads the chunk's counts back; the call returns when the plan
     * is written (its kernels ran on the scheduler's stream).
     * pos_level (device, m entries, or null): the transfers' levels from
     * the host planner, by position in the chunk (1-based; 0 where the
     * event is no valid transfer); the rounds are then skipped.  A level
     * the host left at 0 for a transfer the device finds valid, or a day
     * deeper than the wave keys hold, sends the chunk to the rounds. */
    cudaError_t plan_chunk(long long lo, long long m, int d0, int nd, const long long *bounds,
                           int prev_time, int prev_event, bool has_prev, E2Rec *e2_out,
                           E1Rec *e1_out, int *e1_ptr, int *wave_out, SchedChunk &out,
                           uint32_t *e1_node_out = nullptr, const uint32_t *pos_level = nullptr);

    /* Deepest level the wave keys hold (pos_level above it: the rounds). */
    static int max_host_level();

    /* The E1 records of several chunks (in chunk order, each chunk's by
     * node, with their nodes) as one per-node CSR: stable by node, so each
     * node keeps day and array order.  out holds n records, ptr Nn + 1. */
    cudaError_t merge_e1(const E1Rec *in, const uint32_t *nodes, long long n, E1Rec *out,
                         int *ptr);

    /* Order check and select / shift maxima of events past the last day. */
    cudaError_t check_tail(long long lo, long long m, int prev_time, int prev_event,
                           bool has_prev);

    /* The status so far (order, maxima, planned failures). */
    cudaError_t status(unsigned long long &bad, int &max_select, int &max_shift,
                       std::vector<SchedPlanned> &planned);

    cudaStream_t stream() const { return st_; }

private:
    cudaStream_t st_ = nullptr;
    long long cap_ = 0;
    int Nn_ = 0, nsel_ = 0, nb_ = 1;
    std::vector<void *> bufs_;
    uint8_t *cls_ = nullptr, *jday_ = nullptr;
    uint32_t *s1_ = nullptr, *s2_ = nullptr;
    uint32_t *ks0_ = nullptr, *kd0_ = nullptr, *idx2_ = nullptr, *idx1_ = nullptr;
    uint32_t *ka_ = nullptr, *pa_ = nullptr, *kb_ = nullptr, *pb_ = nullptr;
    uint32_t *ke_ = nullptr, *pe_ = nullptr, *ke2_ = nullptr, *pe2_ = nullptr;
    uint32_t *inv_ = nullptr;
    int *p1_ = nullptr, *p3_ = nullptr, *attach_ = nullptr, *L_ = nullptr, *A_ = nullptr,
        *cnt_ = nullptr;
    uint32_t *hist_ = nullptr;
    unsigned long long *tot_ = nullptr;
    int *dmax_ = nullptr, *deep_ = nullptr;
    int *flags_ = nullptr;
    int *h_flag_ = nullptr;
    long long *info_ = nullptr, *h_info_ = nullptr;    /* device / pinned host */
    SchedStatus *h_status_ = nullptr;                   /* pinned: the status header */
    int *wout_ = nullptr, *h_wout_ = nullptr;          /* compact wave sizes */
    SchedStatus *status_ = nullptr;

    template <class T>
    cudaError_t alloc(T **p, size_t n);
};

/* Per-node offsets ptr[0 .. Nn] of n E1 records whose nodes, keys[0 ..
 * n), are sorted (on stream st). */
cudaError_t e1_ptr_from_keys(const uint32_t *keys, long long n, int Nn, int *ptr,
                             cudaStream_t st);

/* Input range [lo[d], hi[d]) of each day's events (binary search on time).
 * Returns false when the ranges do not tile the table in order, which
 * only an unsorted table can make happen. */
bool event_day_ranges(const siminf_gpu_solver_args *a, const std::vector<DayInfo> &days,
                      std::vector<long long> &lo, std::vector<long long> &hi);

/* Levels of one day's transfers by the host planner, for the days the
 * device leaves to it: the transfers of input range [lo, hi) in wave
 * order into out (returns their count) and the day's wave sizes. */
long long host_day_waves(const int *event, const int *node, const int *dest, const int *n,
                         const double *proportion, const int *select, const int *shift,
                         long long lo, long long hi, int Nn, int nsel, E2Rec *out,
                         std::vector<long long> &waves);

}  // namespace siminf

#endif
