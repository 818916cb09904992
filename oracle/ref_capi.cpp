// C entry points over the reference implementation, for fixture generation
// and for pinning the oracle restatement. Test infrastructure only: this file
// is compiled (by oracle/Makefile, on an x86-64 host with AMX/AVX-512) together
// with the reference's own sources, which it includes in place so that the
// private members and the file-local helpers of src/index.cpp are reachable.
// Nothing in the product links it.
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#define private public
#include "katoann/index.h"
#undef private
#include REF_INDEX_CPP  // the reference's src/index.cpp, path given by the Makefile

namespace {
thread_local std::string g_err;

template <class F>
int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::invalid_argument &e) {
    g_err = e.what();
    return -1;
  } catch (const std::logic_error &e) {
    g_err = e.what();
    return -3;
  } catch (const std::exception &e) {
    g_err = e.what();
    return -2;
  }
}
}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

int ref_build(const float *data, uint32_t n, uint32_t dim, uint32_t nlist, uint32_t train_size,
              uint32_t iters, uint64_t seed, int normalized, uint32_t rotation_sample,
              uint32_t jacobi_sweeps, const char *prefix) {
  return guarded([&] {
    katoann::BuildOptions o;
    o.nlist = nlist;
    o.train_size = train_size;
    o.kmeans_iters = iters;
    o.seed = seed;
    o.normalized = normalized != 0;
    o.rotation_sample = rotation_sample;
    o.jacobi_sweeps = jacobi_sweeps;
    katoann::Index::build(data, n, dim, o, prefix);
  });
}

void *ref_load(const char *prefix, int use_amx, uint32_t prefix_dims, int batched_coarse) {
  auto *idx = new katoann::Index();
  const int rc = guarded([&] {
    katoann::LoadOptions o;
    o.use_amx = use_amx != 0;
    o.prefix_dims = prefix_dims;
    o.batched_coarse = batched_coarse != 0;
    idx->load(prefix, o);
  });
  if (rc) {
    delete idx;
    return nullptr;
  }
  return idx;
}

void ref_free(void *h) { delete static_cast<katoann::Index *>(h); }

// ranking: 0 full, 1 high bytes, 2 prefix. selection: 0 threshold, 1 local.
int ref_search(void *h, const float *q, uint32_t nq, uint32_t k, uint32_t nprobe, int ranking,
               uint32_t survivors, int selection, uint32_t *ids, float *dists) {
  return guarded([&] {
    katoann::SearchParams p;
    p.k = k;
    p.nprobe = nprobe;
    p.ranking = ranking == 0 ? katoann::Ranking::kFull
                : ranking == 1 ? katoann::Ranking::kHighBytes
                               : katoann::Ranking::kPrefix;
    p.survivors = survivors;
    p.selection = selection == 1 ? katoann::Selection::kLocal : katoann::Selection::kThreshold;
    static_cast<const katoann::Index *>(h)->search(q, nq, p, ids, dists);
  });
}

// u32 info[8] = {dim, nlist, npts, dc, head_dims, rotated, engine(0 amx, 1 avx512), batched}
// double scale[4] = {lo, inv_step, step, step_sq}
void ref_info(void *h, uint32_t *info, double *scale) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  info[0] = x.dim_;
  info[1] = x.nlist_;
  info[2] = x.npts_;
  info[3] = x.dc_;
  info[4] = x.head_dims_;
  info[5] = x.rotated_ ? 1u : 0u;
  info[6] = x.engine_ == katoann::Engine::kAmx ? 0u : 1u;
  info[7] = x.coarse_batched_ ? 1u : 0u;
  scale[0] = x.sq_lo_;
  scale[1] = x.sq_inv_step_;
  scale[2] = x.sq_step_;
  scale[3] = x.sq_step_sq_;
}

void ref_list_sizes(void *h, uint32_t *sizes) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  for (uint32_t c = 0; c < x.nlist_; ++c) sizes[c] = static_cast<uint32_t>(x.ids_[c].size());
}

// Unpacks the AMX-packed planes to row-major [rows x dc], lists concatenated in
// list order; also the per-row norms and ids. head_norm is written only when
// the index has a prefix head (else left untouched).
void ref_dump_codes(void *h, uint8_t *hi, uint8_t *lo, int64_t *norm, int64_t *hinorm,
                    int64_t *headnorm, uint32_t *ids) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  const uint32_t Dc = x.dc_, Nc = Dc / 64;
  size_t row = 0;
  for (uint32_t c = 0; c < x.nlist_; ++c) {
    const uint32_t n = static_cast<uint32_t>(x.ids_[c].size());
    for (uint32_t i = 0; i < n; ++i, ++row) {
      for (uint32_t k = 0; k < Dc; ++k) {
        const size_t off = (static_cast<size_t>(i / 16) * Nc + k / 64) * 1024 +
                           (k % 64 / 4) * 64 + (i % 16) * 4 + k % 4;
        hi[row * Dc + k] = x.hi_[c][off];
        lo[row * Dc + k] = x.lo_[c][off];
      }
      norm[row] = x.norm_[c][i];
      hinorm[row] = x.hi_norm_[c][i];
      if (!x.head_norm_.empty()) headnorm[row] = x.head_norm_[c][i];
      ids[row] = x.ids_[c][i];
    }
  }
}

void ref_dump_centroids(void *h, uint8_t *chi, uint8_t *clo, int64_t *cnorm) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  const uint32_t Dc = x.dc_, Nc = Dc / 64;
  for (uint32_t i = 0; i < x.nlist_; ++i) {
    for (uint32_t k = 0; k < Dc; ++k) {
      const size_t off = (static_cast<size_t>(i / 16) * Nc + k / 64) * 1024 +
                         (k % 64 / 4) * 64 + (i % 16) * 4 + k % 4;
      chi[static_cast<size_t>(i) * Dc + k] = x.cen_hi_[off];
      clo[static_cast<size_t>(i) * Dc + k] = x.cen_lo_[off];
    }
    cnorm[i] = x.cen_norm_[i];
  }
}

// The reference's batched rotation (rotate_rows) of nrows x dim rows.
void ref_rotate_rows(void *h, const float *in, uint32_t nrows, float *out) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  katoann::rotate_rows(in, out, nrows, x.dim_, x.rotation_.data());
}

// The reference's per-row rotation used for list vectors (rotate_rows_serial).
void ref_rotate_rows_serial(void *h, const float *in, uint32_t nrows, float *out) {
  const auto &x = *static_cast<const katoann::Index *>(h);
  katoann::rotate_rows_serial(in, out, nrows, x.dim_, x.rotation_.data());
}

// Coarse selection of the reference for already quantized queries (planes
// row-major [nq x dc]); probed is nq x nprobe.
int ref_coarse(void *h, const uint8_t *qhi, const uint8_t *qlo, const int64_t *qnorm,
               uint32_t nq, uint32_t nprobe, uint32_t *probed) {
  return guarded([&] {
    static_cast<const katoann::Index *>(h)->coarse_batched_sq16_(qhi, qlo, qnorm, nq, nprobe,
                                                                  probed);
  });
}

// The public distance kernels (src/kernels.cpp), on AMX-packed planes.
void ref_pack_plane(const uint8_t *rows, uint32_t n, uint32_t dc, uint8_t *out) {
  katoann::pack_plane(rows, n, dc, out);
}
size_t ref_plane_bytes(uint32_t n, uint32_t dc) { return katoann::plane_bytes(n, dc); }
int ref_amx_available() { return katoann::amx_available() ? 1 : 0; }
void ref_sq16_l2(int amx, const uint8_t *qhi, const uint8_t *qlo, const uint8_t *xhi,
                 const uint8_t *xlo, const int64_t *qn, const int64_t *xn, double step_sq,
                 uint32_t m, uint32_t n, uint32_t dc, float *out) {
  katoann::sq16_l2(amx ? katoann::Engine::kAmx : katoann::Engine::kAvx512, qhi, qlo, xhi, xlo,
                   qn, xn, step_sq, m, n, dc, out);
}
void ref_sq16_high_l2(int amx, const uint8_t *qhi, const uint8_t *xhi, const int64_t *qn,
                      const int64_t *xn, double step_sq, uint32_t m, uint32_t n, uint32_t dc,
                      float *out, uint32_t plane_dim) {
  katoann::sq16_high_l2(amx ? katoann::Engine::kAmx : katoann::Engine::kAvx512, qhi, xhi, qn, xn,
                        step_sq, m, n, dc, out, plane_dim);
}

}  // extern "C"
