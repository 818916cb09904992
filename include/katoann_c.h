/* C ABI of libkatoann.so, the host library around katoann::Index. This is the
 * surface a foreign-function binding uses (the Python module binds it with
 * ctypes); it replaces the reference's pybind11 module
 * (python/katoann_module.cpp:34-129) one call for one call. Statuses: 0 ok,
 * -1 invalid argument (std::invalid_argument), -2 runtime error
 * (std::runtime_error, CUDA), -3 logic error (std::logic_error);
 * katoann_last_error() gives the message. Pointers are host memory unless
 * named d_*. */
#ifndef KATOANN_C_H_
#define KATOANN_C_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char *katoann_last_error(void);

/* katoann.amx_available (python/katoann_module.cpp:36-37): always 0 here. */
int katoann_amx_available(void);

/* katoann.build (python/katoann_module.cpp:39-58). */
int katoann_build(const float *data, uint32_t n, uint32_t dim, uint32_t nlist,
                  uint32_t train_size, uint32_t kmeans_iters, uint64_t seed, int normalized,
                  uint32_t rotation_sample, uint32_t jacobi_sweeps, const char *prefix);

void *katoann_index_new(void);
void katoann_index_free(void *index);

/* Index.load (python/katoann_module.cpp:62-76); precision 0 sq16, 1 bf16. */
int katoann_index_load(void *index, const char *prefix, int precision, int use_amx,
                       uint32_t prefix_dims, int batched_coarse, uint32_t max_batch);

/* katoann_index_load through the device-code cache PREFIX.gpucodes
 * (LoadOptions::code_cache): loads the codes when they were made from the
 * same files with the same prefix_dims, else loads the files and writes them. */
int katoann_index_load_cached(void *index, const char *prefix, uint32_t prefix_dims,
                              uint32_t max_batch);

/* Index::save_codes / Index::load_codes: the loaded index as it lives on the
 * device, to and from one file (no counterpart in the reference). */
int katoann_index_save_codes(void *index, const char *path);
int katoann_index_load_codes(void *index, const char *path, uint32_t max_batch);

/* An index from arrays (lists concatenated in list order); on_device selects
 * device pointers for ids, vectors, centroids and rotation. */
int katoann_index_load_arrays(void *index, uint32_t dim, uint32_t nlist, uint32_t npts,
                              int normalized, const float *centroids, const uint32_t *list_sizes,
                              const uint32_t *ids, const float *vectors, const float *rotation,
                              int has_dimc, uint32_t head_dims, int on_device,
                              uint32_t prefix_dims, uint32_t max_batch);

/* Index.search (python/katoann_module.cpp:77-119) without the normalisation,
 * which the caller applies (katoann_normalize_rows). ranking 0 full, 1 high,
 * 2 prefix; selection 0 threshold, 1 local. */
int katoann_index_search(void *index, const float *queries, uint32_t nq, uint32_t k,
                         uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                         uint32_t *ids, float *dists);

/* The same on device memory and a caller stream (cudaStream_t, NULL = the
 * index's stream); asynchronous. timer: katoann_gpu_timer_create() or NULL. */
int katoann_index_search_device(void *index, const float *d_queries, uint32_t nq, uint32_t k,
                                uint32_t nprobe, int ranking, uint32_t survivors, int selection,
                                uint32_t *d_ids, float *d_dists, void *stream, void *timer);

/* info[8] = {dim, nlist, size, prefix_dims, rotated, normalized, batched_coarse, engine=2} */
int katoann_index_info(void *index, uint32_t *info);
size_t katoann_index_memory_bytes(void *index);
int katoann_index_list_sizes(void *index, uint32_t *sizes);
/* [0] coarse boundary ties, [1] survivor boundary ties of the last search. */
int katoann_index_stats(void *index, uint64_t *stats, uint32_t n);
/* The device view (const katoann_gpu_index *) for direct kernel calls. */
const void *katoann_index_device_view(void *index);

/* Unit-length rows as the reference's CLI and module compute them. */
void katoann_normalize_rows(float *rows, size_t n, uint32_t dim);

/* float(double(l2) * step_sq) by the integer method the kernels use. */
float katoann_dist_value(int64_t l2, double step_sq);

#ifdef __cplusplus
}
#endif

#endif /* KATOANN_C_H_ */
