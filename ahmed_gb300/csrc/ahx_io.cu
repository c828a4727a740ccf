// Persistent leaves: the reference's savembls / loadmbls file layout.
//
//   savembls / savembls_   Include/H.h:76-103     mblock::save  Include/mblock.h:737-773
//   loadmbls / loadmbls_   Include/H.h:47-74      mblock::load  Include/mblock.h:775-806
//
// Layout (native byte order; x86-64 and aarch64 agree on it):
//   double eta, uint32 bmin, uint32 nleaves, then per leaf in leaf (DFS) order
//   uint8 present (the reference's bool); if present: uint32 n1, n2, status and
//     status 0 (low rank): uint32 rank, rank*(n1+n2) doubles (U n1 x rank, then V n2 x rank)
//     status 4 (dense):    n1*n2 doubles, column-major
//     status 1 / 5 (Hermitian / symmetric packed): n1*(n1+1)/2 doubles, upper triangle by
//       columns, A(i,j) = data[i + j(j+1)/2] for i <= j (blas::hemva / symva with "U")
//     status 2 / 3: triangular factors of an H-LU; not a product operand, refused.
//
// Save: the leaves sit in the device arena in assembly order, not in leaf order.  Chunks of
// consecutive leaves are gathered into leaf order on the device, copied into pinned host
// memory (two buffers, the next chunk's copy overlapping the current chunk's writes) and
// written record by record.  Load: records are read straight into pinned staging in leaf
// order and uploaded chunk by chunk into a fresh arena, so the loaded arena is in leaf order.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr uint32_t kStatusLowRank = 0, kStatusHerm = 1, kStatusLower = 2, kStatusUpper = 3,
                   kStatusDense = 4, kStatusSym = 5;

// doubles per staging chunk (256 MB); AHX_IO_CHUNK overrides (tests use small chunks)
uint64_t io_chunk() {
  const char* e = std::getenv("AHX_IO_CHUNK");
  if (e && *e) return std::max<uint64_t>(1, std::strtoull(e, nullptr, 10));
  return (uint64_t)32 << 20;
}

struct Gather {
  uint64_t src, dst, count;  // arena offset, chunk offset, doubles
};

// One CTA per leaf: copies the leaf's doubles from the arena into the chunk (leaf order).
__global__ void gather_leaves_kernel(const double* __restrict__ arena, const Gather* __restrict__ g,
                                     double* __restrict__ out) {
  const Gather t = g[blockIdx.x];
  const double* s = arena + t.src;
  double* d = out + t.dst;
  for (uint64_t i = threadIdx.x; i < t.count; i += blockDim.x) d[i] = s[i];
}

struct Pinned {
  double* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
  int alloc(uint64_t n) {
    AHX_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), std::max<uint64_t>(n, 1) * sizeof(double)));
    return AHX_OK;
  }
};

struct Event {
  cudaEvent_t e = nullptr;
  ~Event() {
    if (e) cudaEventDestroy(e);
  }
};

struct OwnedBuf {
  DevBuf b;
  ~OwnedBuf() { b.release(); }
};

uint64_t leaf_count(const Leaf& L, int32_t r) {
  return r < 0 ? (uint64_t)L.n1 * L.n2 : (uint64_t)r * (L.n1 + L.n2);
}

// Sequential writer over the caller's callback; remembers the first failure.
struct Writer {
  ahx_io_fn fn;
  void* ctx;
  bool ok = true;
  void put(const void* p, uint64_t bytes) {
    if (!ok || !bytes) return;
    const int64_t r = fn(ctx, const_cast<void*>(p), bytes);
    if (r < 0 || (uint64_t)r != bytes) ok = false;
  }
  template <class T>
  void put_val(T v) {
    put(&v, sizeof(T));
  }
};

struct Reader {
  ahx_io_fn fn;
  void* ctx;
  bool get(void* p, uint64_t bytes) {
    if (!bytes) return true;
    const int64_t r = fn(ctx, p, bytes);
    return r >= 0 && (uint64_t)r == bytes;
  }
};

int64_t file_write(void* ctx, void* buf, uint64_t bytes) {
  return (int64_t)std::fwrite(buf, 1, bytes, static_cast<std::FILE*>(ctx));
}

int64_t file_read(void* ctx, void* buf, uint64_t bytes) {
  return (int64_t)std::fread(buf, 1, bytes, static_cast<std::FILE*>(ctx));
}

// cplx: the Helmholtz leaves (mblock<dcomp>: two doubles per element; packed
// symmetric diagonal blocks are status 5, SyM) instead of the real ones.
int save_impl(ahx_hmat* H, double eta, uint32_t bmin, Writer& w, bool cplx) {
  if (!(cplx ? H->z.assembled : H->assembled)) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  const std::vector<int32_t>& Rk = cplx ? H->z.rank : H->rank;
  const std::vector<uint64_t>& Of = cplx ? H->z.off : H->off;
  const uint64_t ew = cplx ? 2 : 1;  // doubles per element
  const double* arena = cplx ? H->z.arena.as<double>() : H->arena64.as<double>();
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  w.put_val<double>(eta);
  w.put_val<uint32_t>(bmin);
  w.put_val<uint32_t>(nl);

  // chunks of consecutive leaves, at most `cap` doubles each (a larger leaf gets its own)
  uint64_t total = 0, largest = 0;
  for (uint32_t l = 0; l < nl; ++l) {
    const uint64_t c = leaf_count(Ls[l], Rk[l]) * ew;
    total += c;
    largest = std::max(largest, c);
  }
  const uint64_t cap = std::max(largest, std::min(io_chunk(), std::max<uint64_t>(total, 1)));
  std::vector<Gather> tasks;      // leaves with data, in leaf order
  std::vector<uint32_t> first{0};  // chunk c covers leaves [first[c], first[c+1])
  std::vector<uint32_t> task0{0};  // and tasks [task0[c], task0[c+1])
  {
    uint64_t fill = 0;
    for (uint32_t l = 0; l < nl; ++l) {
      const uint64_t c = leaf_count(Ls[l], Rk[l]) * ew;
      if (fill + c > cap && fill > 0) {
        first.push_back(l);
        task0.push_back((uint32_t)tasks.size());
        fill = 0;
      }
      if (c) tasks.push_back(Gather{Of[l] * ew, fill, c});
      fill += c;
    }
    first.push_back(nl);
    task0.push_back((uint32_t)tasks.size());
  }
  const size_t nchunks = first.size() - 1;

  OwnedBuf dtasks, dstage;
  if ((rc = upload(dtasks.b, tasks, H->stream))) return rc;
  const uint64_t depth = nchunks > 1 ? 2 : 1;
  if ((rc = dstage.b.reserve(depth * cap * sizeof(double)))) return rc;
  Pinned host[2];
  Event ev[2];
  for (uint64_t b = 0; b < depth; ++b) {
    if ((rc = host[b].alloc(cap))) return rc;
    AHX_CUDA(cudaEventCreateWithFlags(&ev[b].e, cudaEventDisableTiming));
  }
  auto enqueue = [&](size_t c) -> int {
    const uint32_t nt = task0[c + 1] - task0[c];
    const uint64_t b = c % depth;
    double* dst = dstage.b.as<double>() + b * cap;
    uint64_t bytes = 0;
    if (nt) {
      const Gather& last = tasks[task0[c + 1] - 1];
      bytes = (last.dst + last.count) * sizeof(double);
      gather_leaves_kernel<<<nt, 256, 0, H->stream>>>(arena, dtasks.b.as<Gather>() + task0[c], dst);
      AHX_CUDA(cudaGetLastError());
      AHX_CUDA(cudaMemcpyAsync(host[b].p, dst, bytes, cudaMemcpyDeviceToHost, H->stream));
    }
    AHX_CUDA(cudaEventRecord(ev[b].e, H->stream));
    return AHX_OK;
  };
  auto write_chunk = [&](size_t c) -> int {
    const uint64_t b = c % depth;
    AHX_CUDA(cudaEventSynchronize(ev[b].e));
    const double* data = host[b].p;
    uint64_t pos = 0;
    for (uint32_t l = first[c]; l < first[c + 1]; ++l) {
      const Leaf& L = Ls[l];
      const int32_t r = Rk[l];
      const uint64_t cnt = leaf_count(L, r) * ew;
      w.put_val<uint8_t>(1);
      w.put_val<uint32_t>(L.n1);
      w.put_val<uint32_t>(L.n2);
      if (r >= 0) {
        w.put_val<uint32_t>(kStatusLowRank);
        w.put_val<uint32_t>((uint32_t)r);
        w.put(data + pos, cnt * sizeof(double));
      } else if (H->tree.sym && L.b1 == L.b2) {
        // diagonal block of a symmetric tree: packed upper triangle (Hermitian for
        // real leaves, complex symmetric for the Helmholtz ones)
        w.put_val<uint32_t>(cplx ? kStatusSym : kStatusHerm);
        for (uint32_t j = 0; j < L.n1; ++j)
          w.put(data + pos + (uint64_t)j * L.n1 * ew, (uint64_t)(j + 1) * ew * sizeof(double));
      } else {
        w.put_val<uint32_t>(kStatusDense);
        w.put(data + pos, cnt * sizeof(double));
      }
      pos += cnt;
    }
    return AHX_OK;
  };
  if (nchunks && (rc = enqueue(0))) return rc;
  for (size_t c = 0; c < nchunks; ++c) {
    // the next chunk's gather and copy run while this chunk is written
    if (c + 1 < nchunks && (rc = enqueue(c + 1))) return rc;
    if ((rc = write_chunk(c))) return rc;
    if (!w.ok) break;
  }
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  if (!w.ok) {
    set_error("savembls: write failed");
    return AHX_ERR_ARG;
  }
  return AHX_OK;
}

// Stages leaf data in leaf order into pinned buffers and uploads them into the arena.
struct Stager {
  ahx_hmat* H;
  bool cplx;  // the Helmholtz arena (offsets in doubles: two per element)
  uint64_t cap;
  Pinned buf[2];
  Event ev[2];
  int cur = 0;
  uint64_t fill = 0, base = 0;  // staged doubles and the arena offset of buf[cur][0]
  bool used[2] = {false, false};

  int init(uint64_t c) {
    cap = c;
    int rc;
    for (int b = 0; b < 2; ++b) {
      if ((rc = buf[b].alloc(cap))) return rc;
      AHX_CUDA(cudaEventCreateWithFlags(&ev[b].e, cudaEventDisableTiming));
    }
    return AHX_OK;
  }
  int flush() {
    if (fill) {
      double* arena = cplx ? H->z.arena.as<double>() : H->arena64.as<double>();
      AHX_CUDA(cudaMemcpyAsync(arena + base, buf[cur].p, fill * sizeof(double), cudaMemcpyHostToDevice, H->stream));
      AHX_CUDA(cudaEventRecord(ev[cur].e, H->stream));
      used[cur] = true;
      base += fill;
      fill = 0;
      cur ^= 1;
      if (used[cur]) AHX_CUDA(cudaEventSynchronize(ev[cur].e));  // its upload is done
    }
    return AHX_OK;
  }
  // room for up to `want` doubles at the end of the staged data (flushes when full)
  int room(uint64_t want, double*& p, uint64_t& got) {
    if (fill == cap) {
      int rc = flush();
      if (rc) return rc;
    }
    got = std::min(want, cap - fill);
    p = buf[cur].p + fill;
    return AHX_OK;
  }
};

int load_impl(ahx_hmat* H, Reader& rd, double* eta_out, uint32_t* bmin_out, bool cplx) {
  double eta = 0.0;
  uint32_t bmin = 0, nfile = 0;
  if (!rd.get(&eta, sizeof eta) || !rd.get(&bmin, sizeof bmin) || !rd.get(&nfile, sizeof nfile)) {
    set_error("loadmbls: truncated header");
    return AHX_ERR_ARG;
  }
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  if (nfile != nl) {
    set_error("loadmbls: the file holds " + std::to_string(nfile) +
              " leaves, the block-cluster tree " + std::to_string(nl));
    return AHX_ERR_ARG;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  const uint64_t ew = cplx ? 2 : 1;  // doubles per element
  // capacity estimate: dense inadmissible leaves plus 16 columns per admissible leaf
  uint64_t est = 0;
  for (const Leaf& L : Ls)
    est += L.adm ? (uint64_t)(L.n1 + L.n2) * 16 : (uint64_t)L.n1 * L.n2;
  if (cplx) {
    ZState& Z = H->z;
    Z.assembled = Z.valid32 = Z.table = false;
    Z.k = Z.h = Z.eps = 0.0;
    Z.elems = 0;
    Z.arena.release();
    if ((rc = Z.arena.reserve(std::max<uint64_t>(est, 1) * ew * sizeof(double)))) return rc;
  } else {
    invalidate_products(H);
    H->assembled = false;
    H->h = H->eps = 0.0;
    H->arena64_elems = 0;
    H->arena64.release();
    if ((rc = H->arena64.reserve(std::max<uint64_t>(est, 1) * sizeof(double)))) return rc;
  }
  std::vector<int32_t> rank(nl, 0);
  std::vector<uint64_t> off(nl, 0);
  Stager st{H, cplx};
  if ((rc = st.init(std::min(io_chunk(), std::max<uint64_t>(est, 1 << 16))))) return rc;
  std::vector<double> packed, full;
  auto fail = [&](const std::string& msg) {
    set_error("loadmbls: leaf " + msg);
    return AHX_ERR_ARG;
  };
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    uint8_t present = 0;
    if (!rd.get(&present, 1)) return fail(std::to_string(l) + ": truncated");
    if (present > 1) return fail(std::to_string(l) + ": corrupt presence flag");
    uint32_t n1 = L.n1, n2 = L.n2, status = kStatusLowRank, r = 0;
    if (present) {
      if (!rd.get(&n1, 4) || !rd.get(&n2, 4) || !rd.get(&status, 4))
        return fail(std::to_string(l) + ": truncated");
      if (n1 != L.n1 || n2 != L.n2)
        return fail(std::to_string(l) + ": " + std::to_string(n1) + " x " + std::to_string(n2) +
                    " in the file, " + std::to_string(L.n1) + " x " + std::to_string(L.n2) +
                    " in the block-cluster tree");
      if (status == kStatusLowRank) {
        if (!rd.get(&r, 4)) return fail(std::to_string(l) + ": truncated");
        if ((uint64_t)r > (uint64_t)n1 + n2) return fail(std::to_string(l) + ": rank out of range");
      } else if (status == kStatusLower || status == kStatusUpper) {
        return fail(std::to_string(l) + ": triangular (H-LU factor) blocks are not product operands");
      } else if (status == kStatusHerm || status == kStatusSym) {
        if (n1 != n2) return fail(std::to_string(l) + ": packed block is not square");
      } else if (status != kStatusDense) {
        return fail(std::to_string(l) + ": unknown status " + std::to_string(status));
      }
    }
    // a missing block (present = 0) is a zero block: rank 0
    const bool dense = present && status != kStatusLowRank;
    rank[l] = dense ? -1 : (int32_t)r;
    const uint64_t cnt_el = dense ? (uint64_t)n1 * n2 : (uint64_t)r * (n1 + n2);
    const uint64_t cnt = cnt_el * ew;  // doubles
    if ((rc = cplx ? zarena_append(H, cnt_el, off[l]) : arena_append(H, cnt_el, off[l]))) return rc;
    if (dense && status != kStatusDense) {
      // expand the packed upper triangle: symmetric (SyM; real Hermitian), or
      // Hermitian for complex data (the mirror conjugated)
      const bool conj = cplx && status == kStatusHerm;
      packed.resize((uint64_t)n1 * (n1 + 1) / 2 * ew);
      if (!rd.get(packed.data(), packed.size() * sizeof(double)))
        return fail(std::to_string(l) + ": truncated");
      full.assign(cnt, 0.0);
      for (uint32_t j = 0; j < n1; ++j)
        for (uint32_t i = 0; i <= j; ++i)
          for (uint64_t c = 0; c < ew; ++c) {
            const double v = packed[(i + (uint64_t)j * (j + 1) / 2) * ew + c];
            full[(i + (uint64_t)j * n1) * ew + c] = v;
            if (i != j) full[(j + (uint64_t)i * n1) * ew + c] = conj && c == 1 ? -v : v;
          }
      for (uint64_t done = 0; done < cnt;) {
        double* p;
        uint64_t got;
        if ((rc = st.room(cnt - done, p, got))) return rc;
        std::memcpy(p, full.data() + done, got * sizeof(double));
        st.fill += got;
        done += got;
      }
    } else {
      for (uint64_t done = 0; done < cnt;) {
        double* p;
        uint64_t got;
        if ((rc = st.room(cnt - done, p, got))) return rc;
        if (!rd.get(p, got * sizeof(double))) return fail(std::to_string(l) + ": truncated");
        st.fill += got;
        done += got;
      }
    }
  }
  if ((rc = st.flush())) return rc;
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  if (cplx) {
    H->z.rank = rank;
    H->z.aca_rank = rank;
    H->z.off = off;
    H->z.assembled = true;
  } else {
    H->rank = rank;
    H->aca_rank = rank;
    H->off = off;
    H->assembled = true;
  }
  if (eta_out) *eta_out = eta;
  if (bmin_out) *bmin_out = bmin;
  return AHX_OK;
}

}  // namespace
}  // namespace ahx

using namespace ahx;

extern "C" {

int ahx_mbls_header(const char* path, double* eta, uint32_t* bmin, uint32_t* nleaves) {
  if (!path) return AHX_ERR_ARG;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error(std::string("loadmbls: cannot open ") + path);
    return AHX_ERR_ARG;
  }
  double e = 0.0;
  uint32_t b = 0, n = 0;
  const bool ok = std::fread(&e, sizeof e, 1, f) == 1 && std::fread(&b, sizeof b, 1, f) == 1 &&
                  std::fread(&n, sizeof n, 1, f) == 1;
  std::fclose(f);
  if (!ok) {
    set_error("loadmbls: truncated header");
    return AHX_ERR_ARG;
  }
  if (eta) *eta = e;
  if (bmin) *bmin = b;
  if (nleaves) *nleaves = n;
  return AHX_OK;
}

}  // extern "C"

namespace {
int save_path(ahx_hmat* H, double eta, uint32_t bmin, const char* path, bool cplx) {
  if (!H || !path) return AHX_ERR_ARG;
  std::FILE* f = std::fopen(path, "wb");
  if (!f) {
    set_error(std::string("savembls: cannot open ") + path);
    return AHX_ERR_ARG;
  }
  std::vector<char> iobuf(1 << 20);
  std::setvbuf(f, iobuf.data(), _IOFBF, iobuf.size());
  Writer w{file_write, f};
  int rc = save_impl(H, eta, bmin, w, cplx);
  if (std::fclose(f) != 0 && rc == AHX_OK) {
    set_error("savembls: write failed");
    rc = AHX_ERR_ARG;
  }
  return rc;
}

int load_path(ahx_hmat* H, const char* path, double* eta, uint32_t* bmin, bool cplx) {
  if (!H || !path) return AHX_ERR_ARG;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error(std::string("loadmbls: cannot open ") + path);
    return AHX_ERR_ARG;
  }
  std::vector<char> iobuf(1 << 20);
  std::setvbuf(f, iobuf.data(), _IOFBF, iobuf.size());
  Reader rd{file_read, f};
  const int rc = load_impl(H, rd, eta, bmin, cplx);
  std::fclose(f);
  return rc;
}
}  // namespace

extern "C" {

int ahx_hmat_save_stream(ahx_hmat* H, double eta, uint32_t bmin, ahx_io_fn write, void* ctx) {
  if (!H || !write) return AHX_ERR_ARG;
  Writer w{write, ctx};
  return save_impl(H, eta, bmin, w, false);
}

int ahx_hmat_load_stream(ahx_hmat* H, ahx_io_fn read, void* ctx, double* eta, uint32_t* bmin) {
  if (!H || !read) return AHX_ERR_ARG;
  Reader rd{read, ctx};
  return load_impl(H, rd, eta, bmin, false);
}

int ahx_hmat_save(ahx_hmat* H, double eta, uint32_t bmin, const char* path) {
  return save_path(H, eta, bmin, path, false);
}

int ahx_hmat_load(ahx_hmat* H, const char* path, double* eta, uint32_t* bmin) {
  return load_path(H, path, eta, bmin, false);
}

int ahx_helm_save_stream(ahx_hmat* H, double eta, uint32_t bmin, ahx_io_fn write, void* ctx) {
  if (!H || !write) return AHX_ERR_ARG;
  Writer w{write, ctx};
  return save_impl(H, eta, bmin, w, true);
}

int ahx_helm_load_stream(ahx_hmat* H, ahx_io_fn read, void* ctx, double* eta, uint32_t* bmin) {
  if (!H || !read) return AHX_ERR_ARG;
  Reader rd{read, ctx};
  return load_impl(H, rd, eta, bmin, true);
}

int ahx_helm_save(ahx_hmat* H, double eta, uint32_t bmin, const char* path) {
  return save_path(H, eta, bmin, path, true);
}

int ahx_helm_load(ahx_hmat* H, const char* path, double* eta, uint32_t* bmin) {
  return load_path(H, path, eta, bmin, true);
}

}  // extern "C"
