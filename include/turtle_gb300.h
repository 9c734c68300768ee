/*
 * turtle_gb300.h -- C ABI of the GB300 (sm_103a) TurtleSort sort path.
 *
 * Plain C: no CUDA, C++ or torch types.  Streams are passed as `void*`
 * (a cudaStream_t; NULL = the handle's own stream).  Every entry point
 * returns a turtle_status (0 = success) and never exits the process.
 *
 * Each declaration names the reference interface it replaces
 * (tugrul512bit/TurtleSort, file:line).
 */
#ifndef TURTLE_GB300_H
#define TURTLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Key types.  The reference instantiates its kernels for char, unsigned
 * char, short, unsigned short, int, unsigned, long, unsigned long
 * (turtle-sort.cu:956-1134); these are the same eight integer types.  It also
 * instantiates float and double (turtle-sort.cu:1136-1174), compared with <
 * so that NaN placement is undefined; here they sort in IEEE-754 totalOrder:
 * -NaN < -inf < ... < -0.0 < +0.0 < ... < +inf < +NaN, ties (equal bit
 * patterns) in input order. */
typedef enum turtle_dtype {
  TURTLE_INT8 = 0,
  TURTLE_UINT8 = 1,
  TURTLE_INT16 = 2,
  TURTLE_UINT16 = 3,
  TURTLE_INT32 = 4,
  TURTLE_UINT32 = 5,
  TURTLE_INT64 = 6,
  TURTLE_UINT64 = 7,
  TURTLE_FLOAT32 = 8,
  TURTLE_FLOAT64 = 9
} turtle_dtype;

/* Status codes.  The reference aborts the process on any CUDA error
 * (turtle-globals.cuh:18-30, gpuErrchk -> exit) and prints device-side errors
 * (turtle-sort.cu:146,608,859); these codes replace both. */
typedef enum turtle_status {
  TURTLE_OK = 0,
  TURTLE_ERR_INVALID_ARGUMENT = 1, /* null handle/pointer, bad dtype, n < 0 */
  TURTLE_ERR_TOO_LARGE = 2,        /* n (or arrays x size) above the handle's max_n */
  TURTLE_ERR_CUDA = 3,             /* a CUDA runtime/driver call failed */
  TURTLE_ERR_OUT_OF_MEMORY = 4,    /* device or pinned allocation failed */
  TURTLE_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up */
  TURTLE_ERR_CAPACITY = 6,         /* a device work list would have overflowed */
  TURTLE_ERR_STATE = 7,            /* e.g. Sync without StartSorting */
  TURTLE_ERR_ALIGNMENT = 8,        /* device pointer not 16-byte aligned */
  TURTLE_ERR_NO_DEVICE = 9,        /* no usable CUDA device */
  TURTLE_ERR_BUDGET = 10           /* a request can never fit the HBM budget */
} turtle_status;

typedef struct turtle_sorter turtle_sorter; /* opaque */

/* ---- the drop-in sorter (turtle-sort.cuh:31-283, struct TurtleSort) ---- */

/* Replaces TurtleSort(int maxElements, bool optInCompression)
 * (turtle-sort.cuh:63-113): device buffers for up to max_n keys (+ int32
 * index when track_index != 0), a private stream, and the work lists of the
 * persistent sort kernel.  Buffers come from the CUDA driver VMM API; with
 * compress != 0 they request generic compression when the device supports it
 * (turtle-buffer.cuh:27-70, quick-helper.cuh:57-105).  device < 0 means the
 * current device (the reference hard-codes device 0, turtle-sort.cuh:73). */
turtle_status turtle_create(turtle_dtype dtype, int64_t max_n, int track_index, int compress,
                            int device, turtle_sorter** out);

/* Replaces ~TurtleSort (turtle-sort.cuh:278-282) and the Buffer destructors
 * (turtle-buffer.cuh:82-99).  Safe on NULL. */
turtle_status turtle_destroy(turtle_sorter* s);

/* Replaces MemoryCompressionSuccessful() (turtle-sort.cuh:115-118): 1 when
 * the key buffers really were allocated compressible. */
int turtle_compression_ok(const turtle_sorter* s);

/* Replaces StartSorting(std::vector<Type>*, std::vector<int>*)
 * (turtle-sort.cuh:124-184): copies n keys (and n int32 ids when idx is not
 * NULL) from host memory and starts the sort asynchronously.  The host
 * buffers must stay valid until turtle_sync returns; results are written back
 * into them by the time turtle_sync returns.  When both buffers are pinned
 * (cudaHostAlloc / cudaHostRegister) and n >= 4M, the result is copied back
 * slice by slice while the rest of the array is still being sorted; the
 * buffers' contents are then unspecified if turtle_sync reports an error. */
turtle_status turtle_start(turtle_sorter* s, void* host_keys, int32_t* host_idx, int64_t n);

/* Replaces double Sync() (turtle-sort.cuh:188-258): waits for the sort,
 * copies keys (and ids) back into the buffers given to turtle_start and
 * stores the seconds elapsed since turtle_start in *seconds (may be NULL). */
turtle_status turtle_sync(turtle_sorter* s, double* seconds);

/* Replaces MultiSort<Type,ArrSize,BlockSize,UseSharedMemory>(numArrays, ptr)
 * (turtle-sort.cuh:265-276 -> turtle-multi-sort.cuh:195-205): sorts
 * num_arrays contiguous arrays of arr_size keys in place in host memory,
 * synchronously.  block_size is accepted for source compatibility and only
 * checked the way the reference requires (num_arrays % block_size == 0).
 * num_arrays * arr_size must not exceed max_n.  *seconds (may be NULL)
 * receives the wall time including both copies, like the reference. */
turtle_status turtle_multisort(turtle_sorter* s, void* host_keys, int64_t arr_size,
                               int64_t num_arrays, int block_size, double* seconds);

/* MultiSort with an id per key (the reference's MultiSort has none,
 * README.md:46): as turtle_multisort, and host_idx (num_arrays * arr_size
 * int32) is permuted with the keys, each array's ids in the stable order of
 * its keys.  Needs a sorter created with track_index != 0. */
turtle_status turtle_multisort_idx(turtle_sorter* s, void* host_keys, int32_t* host_idx,
                                   int64_t arr_size, int64_t num_arrays, int block_size,
                                   double* seconds);

/* ---- device-resident forms (no reference counterpart; new API) ---- */

/* Sorts n keys (and ids) that are already in device memory, in place, on
 * `stream` (NULL = the sorter's stream).  Asynchronous: call
 * turtle_stream_status (or synchronize the stream) before reading results. */
turtle_status turtle_sort_device(turtle_sorter* s, void* d_keys, int32_t* d_idx, int64_t n,
                                 void* stream);

/* Batched uneven form: num arrays packed back to back in d_keys (and d_idx),
 * array i = [offsets[i], offsets[i+1]), offsets in device memory (num + 1
 * int64 values, offsets[0] = 0, non-decreasing, offsets[num] <= max_n).
 * All arrays are sorted by one persistent launch; the launch is captured in a
 * CUDA graph the first time a given (pointers, num, total) is seen and
 * replayed afterwards.  Asynchronous like turtle_sort_device. */
turtle_status turtle_sort_batched_device(turtle_sorter* s, void* d_keys, int32_t* d_idx,
                                         const int64_t* d_offsets, int64_t num, int64_t total,
                                         void* stream);

/* Fixed-size batched form on device memory: num_arrays arrays of arr_size
 * keys (one CTA or thread group per array, shared-memory sort).  Arrays
 * longer than the shared-memory capacity go through the batched persistent
 * path.  Asynchronous. */
turtle_status turtle_multisort_device(turtle_sorter* s, void* d_keys, int32_t* d_idx,
                                      int64_t arr_size, int64_t num_arrays, void* stream);

/* Waits for the work issued on `stream` (NULL = the sorter's stream) and
 * returns the device-side status of the last sort on this sorter
 * (TURTLE_OK, TURTLE_ERR_TIMEOUT, TURTLE_ERR_CAPACITY). */
turtle_status turtle_stream_status(turtle_sorter* s, void* stream);

/* Allocation-free sort (no counterpart in the reference): for callers that
 * may not allocate device memory when they sort -- hosts that own a fixed
 * device-memory pool and forbid allocations after start-up, plugins handed
 * device pointers but no allocator, real-time loops that must not block on
 * the allocator.  Sorts n keys (and ids, or NULL) already in device memory, in
 * place, on `stream` (NULL = the legacy default stream), using only a 16 MiB
 * scratch array compiled into the library (held by every GPU that loads the
 * library until exit).  n must not exceed turtle_noalloc_max_elements()
 * (1,048,576), else TURTLE_ERR_TOO_LARGE; pointers must be 16-byte aligned.
 * All calls share the scratch array: calls whose work overlaps on the GPU
 * race and corrupt each other.  The first call on a device looks up the
 * array's address and prepares the kernels.  Waits for `stream` and returns
 * the device-side status.  Calls no allocating routine. */
turtle_status turtle_sort_device_noalloc(turtle_dtype dtype, void* d_keys, int32_t* d_idx,
                                         int64_t n, void* stream);

/* Largest n accepted by turtle_sort_device_noalloc. */
int64_t turtle_noalloc_max_elements(void);

/* ---- serving loop: continuous batching (no reference counterpart) ----
 *
 * The reference sorts one array per StartSorting/Sync pair on one host thread
 * (turtle-sort.cuh:124-258); a serving process calls it once per request,
 * serially.  A turtle_server takes requests of any of the eight dtypes, with
 * or without ids, from any host thread.  A scheduler thread admits waiting
 * requests while their device memory fits the HBM budget: the oldest waiting
 * request opens a batch and the requests of its (dtype, ids) group among the
 * next 256 waiting ones join it, in one batched persistent launch; a request
 * of at least 2^20 keys is sorted alone, as a plain sort.  Up to
 * eight batches are in flight: copies in and out overlap other batches'
 * sorts, and two batches sort at once, each on half of the GPU.  Results are
 * identical to sorting each request alone. */
typedef struct turtle_server turtle_server; /* opaque */

typedef struct turtle_server_stats {
  int64_t submitted, completed, failed, batches;
  int64_t keys;          /* keys of completed requests */
  double p50_ms, p99_ms, mean_ms, max_ms; /* submit -> done latency */
  double span_s;         /* first submit -> last completion */
  double keys_per_s;     /* keys / span_s */
  int64_t in_use_bytes;  /* device bytes held by batches in flight */
} turtle_server_stats;

/* Starts a server on `device` (< 0: current) that holds at most
 * hbm_budget_bytes of device memory for batches in flight.  A batch fuses at
 * most max_batch_requests requests (<= 0: 4096) and max_batch_keys keys
 * (<= 0: 2^25; at most 2^31 - 1; a single larger request forms a batch
 * alone). */
turtle_status turtle_server_create(int device, int64_t hbm_budget_bytes, int max_batch_requests,
                                   int64_t max_batch_keys, turtle_server** out);

/* Queues a sort of n keys at host_keys (and n int32 ids at host_idx, or NULL)
 * in place.  Host buffers should be pinned for full copy speed and must stay
 * valid until turtle_server_wait returns for the ticket.  A request whose
 * batch can never fit the budget completes with TURTLE_ERR_BUDGET. */
turtle_status turtle_server_submit(turtle_server* srv, turtle_dtype dtype, void* host_keys,
                                   int32_t* host_idx, int64_t n, uint64_t* ticket);

/* *done = 1 when the request has finished (results are in its buffers). */
turtle_status turtle_server_poll(turtle_server* srv, uint64_t ticket, int* done);

/* Blocks until the request has finished, stores its submit-to-done latency
 * (may be NULL), releases the ticket and returns the request's status. */
turtle_status turtle_server_wait(turtle_server* srv, uint64_t ticket, double* latency_seconds);

/* Blocks until no request is waiting or in flight. */
turtle_status turtle_server_drain(turtle_server* srv);

/* Counters and latency percentiles of the completed requests. */
turtle_status turtle_server_get_stats(turtle_server* srv, turtle_server_stats* out);

/* Finishes every queued request, then stops the scheduler thread and frees
 * the server.  Safe on NULL. */
turtle_status turtle_server_destroy(turtle_server* srv);

/* Pivot rule of this sorter (no counterpart in the reference; the output is
 * the same whichever rule runs because every step is stable):
 *   TURTLE_PIVOTS_REFERENCE  sorted{a[start+n/2], a[start], a[stop]} per
 *                            segment, as the reference (turtle-sort.cu:641-655);
 *   TURTLE_PIVOTS_SAMPLED    the quartiles of 31 evenly spaced keys of the
 *                            segment: fewer partition levels;
 *   TURTLE_PIVOTS_TWO_LEVEL  passes that apply two levels at once (31 classes;
 *                            pivots from 63 evenly spaced keys): half the
 *                            passes over the data, more work per key;
 *   TURTLE_PIVOTS_AUTO       (default) the tuned table's form for the key
 *                            type and size;
 *   TURTLE_FORM_RADIX        no pivots: least-significant-digit radix passes
 *                            over 8-bit digits (one read + one write of keys
 *                            and ids per digit that varies, plus one histogram
 *                            read); batched sorts keep a pivot form. */
#define TURTLE_PIVOTS_REFERENCE 0
#define TURTLE_PIVOTS_SAMPLED 1
#define TURTLE_PIVOTS_TWO_LEVEL 2
#define TURTLE_PIVOTS_AUTO 3
#define TURTLE_FORM_RADIX 4
turtle_status turtle_set_pivot_rule(turtle_sorter* s, int rule);

/* ---- introspection ---- */

/* Kernel launches issued by this sorter since it was created. */
int64_t turtle_launch_count(const turtle_sorter* s);

/* Partition levels run by the last completed sort (after turtle_stream_status
 * or turtle_sync). */
int turtle_last_levels(const turtle_sorter* s);

/* Form of the last enqueued sort: TURTLE_FORM_RADIX, or the pivot rule its
 * partition used (TURTLE_PIVOTS_REFERENCE / _SAMPLED / _TWO_LEVEL); for the
 * radix form turtle_last_levels is the number of digit passes that moved
 * keys. */
int turtle_last_form(const turtle_sorter* s);

/* Largest n a sorter of this dtype can be created for (limited by the int32
 * index payload when track_index != 0). */
int64_t turtle_max_elements(turtle_dtype dtype, int track_index);

/* Element capacity of the one-CTA shared-memory sort for this dtype: arrays
 * up to this length are sorted without a partition pass. */
int64_t turtle_smem_capacity(turtle_dtype dtype, int track_index);

/* Short text for a status code (static storage). */
const char* turtle_status_string(turtle_status st);

/* Text of the last CUDA error seen by this sorter ("" if none). */
const char* turtle_last_cuda_error(const turtle_sorter* s);

/* Host-side fault injection for tests: the next `count` device-buffer
 * allocations fail as if the device were out of memory.  No GPU fault is
 * involved; callers see TURTLE_ERR_OUT_OF_MEMORY. */
void turtle_debug_fail_allocations(int count);

/* Like turtle_debug_fail_allocations, but only the k-th device-buffer
 * allocation from now on fails (k = 1: the next one) and the ones before it
 * succeed, so a test can fail a constructor part-way and check that nothing
 * it had allocated stays behind.  0 cancels. */
void turtle_debug_fail_allocation_at(int k);

/* Phase timeline of the last persistent-kernel sort (valid after
 * turtle_stream_status / turtle_sync): globaltimer nanoseconds taken after
 * each grid barrier, with the work items of the phase that ended there, and a
 * final entry (info = -2) when the last CTA finished.  Returns the number of
 * entries written (at most max). */
int turtle_debug_timeline(const turtle_sorter* s, uint64_t* ns, int32_t* info, int max);

/* Kernel timing for measurement: with enable != 0, every later sort on this
 * sorter records CUDA events on its launch stream before the partition
 * kernel, between it and the leaf kernel, and after the leaf kernel (graph-
 * captured batched sorts excepted).  Resets the count of timed sorts. */
turtle_status turtle_debug_time_kernels(turtle_sorter* s, int enable);

/* Sums over the last `last` timed sorts (at most 64) of the partition
 * kernel's and the leaf kernel's durations in milliseconds; waits for those
 * sorts.  Returns the number of sorts summed (0 if timing is off). */
int turtle_debug_kernel_times(turtle_sorter* s, int last, double* partition_ms, double* leaf_ms);

/* The partition time of the same sorts split at the start of the partition
 * kernel (radix form: of the first digit pass): setup_ms = before it (float
 * map; radix: histogram and plan kernels), pass_ms = the partition kernel
 * (radix: all digit-pass kernels).  For the radix form partition_ms above
 * covers histogram, plan and passes, leaf_ms the finish kernel. */
int turtle_debug_pass_times(turtle_sorter* s, int last, double* setup_ms, double* pass_ms);

/* Where the last sort's device-side error was recorded (valid after
 * turtle_stream_status / turtle_sync): site 1 = grid barrier wait limit,
 * 2 = grid barrier (with leaf work) wait limit, 3 = bulk-copy wait limit,
 * 4 = a work list was full, 5 = radix look-back wait limit (info = the tile
 * that gave up); block = the CTA; info = site detail.  Returns
 * the device status word (0 = no error). */
int turtle_debug_error_site(const turtle_sorter* s, int* site, int* block, int* info);

/* For testing the yield path: later sorts on this sorter stop the partition
 * and drain the leaf lists (leaf launches, then a resumed partition) whenever
 * more than `leaves` leaves are pending at the start of a level.  0 restores
 * the default (yield only when the lists could overflow). */
turtle_status turtle_debug_yield_threshold(turtle_sorter* s, int32_t leaves);

/* For testing the bounded device-side waits (no counterpart in the
 * reference, whose CDP kernels have no waits of their own): later sorts on
 * this sorter give up a grid-barrier wait after `polls` polls instead of the
 * default limit (about a second of polling), record TURTLE_ERR_TIMEOUT and
 * return, leaving the context usable.  0 restores the default.  Only the
 * grid-barrier wait is shortened; a CTA has no bulk copy in flight there. */
turtle_status turtle_debug_barrier_polls(turtle_sorter* s, int64_t polls);

/* Testing the radix form's bounded look-back wait: tile `tile` (>= 0) of every
 * later radix-form digit pass never publishes its look-back words, so the
 * tiles after it wait until the poll limit (turtle_debug_barrier_polls) and
 * the sort reports TURTLE_ERR_TIMEOUT without writing; tile < 0 turns it off.
 * The GPU stays usable: no wait is unbounded and nothing faults. */
turtle_status turtle_debug_radix_stall(turtle_sorter* s, int64_t tile);

/* ---- launch configuration (autotuning) ----
 *
 * The reference fixes its kernel geometry at compile time
 * (turtle-sort.cu:7,12; MultiSort's ArrSize / BlockSize template parameters,
 * turtle-multi-sort.cuh:11,13).  Here each sort picks, by key type, index
 * flag and size band, a configuration from a table that the project's tuner
 * (turtlesort_gb300/tune.py) measured on the GPU and compiled into the
 * library: pass form (TURTLE_PIVOTS_SAMPLED one-level,
 * TURTLE_PIVOTS_TWO_LEVEL or TURTLE_FORM_RADIX), partition tile (1 << tile_shift keys, shift
 * 10..12), shared-memory sort geometry (0..3, see turtle_leaf_geometry), leaf
 * cut (segments of at most leaf_cut keys are sorted in shared memory; 1024 up
 * to the geometry's capacity) and partition grid (resident CTAs / grid_div,
 * grid_div 1, 2 or 4).  The output never depends on the configuration. */

/* enable != 0 (default): sorts use the tuned table; 0: the compile-time
 * defaults (the configuration before tuning). */
turtle_status turtle_set_tuning(turtle_sorter* s, int enable);

/* Pins one configuration for every later sort on this sorter (form < 0
 * returns to the table; form TURTLE_FORM_RADIX: plain sorts use the radix
 * form, batched sorts two-level passes with the other values).  May reallocate the sorter's work lists, after
 * waiting for the device.  TURTLE_ERR_INVALID_ARGUMENT for values outside the
 * ranges above. */
turtle_status turtle_set_config(turtle_sorter* s, int form, int tile_shift, int leaf_geometry,
                                int leaf_cut, int grid_div);

/* The table's configuration for n keys: out6 = {form, tile_shift,
 * leaf_geometry, leaf_cut, grid_div, radix}; radix = 1 when plain sorts of
 * that size use TURTLE_FORM_RADIX (the other values then configure batched
 * sorts). */
turtle_status turtle_tuning_lookup(turtle_dtype dtype, int track_index, int64_t n, int32_t* out6);

/* The table's shared-memory geometry for MultiSort arrays of arr_size keys
 * (-1: none listed; the default geometry is used). */
int turtle_tuning_multisort_geometry(turtle_dtype dtype, int track_index, int64_t arr_size);

/* Where the table came from (device, date), static storage. */
const char* turtle_tuning_source(void);

/* Shared-memory sort geometry g (0..3) for this key type: out4 = {CTA
 * threads, keys per thread, capacity, size classes}.  Returns 0 for bad
 * arguments. */
int turtle_leaf_geometry(turtle_dtype dtype, int geometry, int32_t* out4);

/* For the tuner and tests: MultiSort of num_arrays arrays of arr_size keys in
 * device memory with shared-memory geometry `geometry` (no sorter needed;
 * asynchronous on `stream`, NULL = the legacy default stream).
 * TURTLE_ERR_TOO_LARGE when the arrays exceed the geometry's capacity. */
turtle_status turtle_debug_multisort_geometry(turtle_dtype dtype, void* d_keys, int32_t* d_idx,
                                              int64_t arr_size, int64_t num_arrays, int geometry,
                                              void* stream);

/* Library version string (static storage). */
const char* turtle_version(void);

#ifdef __cplusplus
}
#endif

#endif /* TURTLE_GB300_H */
