// wtg_fm.cu -- FM-index counting on the GPU: backward search over the wavelet
// tree of a BWT.
//
// The reference builds the FM-index -- suffix array by divsufsort, the BWT
// s[SA[i]-1] (s[n-1] where SA[i] == 0), a wavelet tree over it
// (fm-index/par/WT.C:33-45) -- and stops there.  Counting is the standard
// backward search: [sp, ep) = [0, n), then for the pattern's symbols from the
// last to the first  sp = C[c] + rank(sp, c),  ep = C[c] + rank(ep, c), where
// rank is wt_int's (wt_int/wt_int_par.hpp:553-577) over the tree of the BWT
// and C[c] counts the symbols below c.
//
// The path of a symbol through the tree does not depend on the position, so
// each symbol's node offsets and ones-before counts are tabulated once per
// call (fm_paths_kernel); a rank then costs one rank_support_v probe per
// level, and sp and ep share the path.
#include "wtg_select.cuh"
#include "wtg_tree.cuh"

namespace wtg {
namespace {

// paths[c * L + l] = (global bit offset of c's node at level l, ones before it)
__global__ void fm_paths_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt, uint64_t n,
                                int L, uint64_t sigma, ulonglong2* __restrict__ paths) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= sigma) return;
  uint64_t offset = 0, size = n;
  for (int l = 0; l < L; ++l) {
    const uint64_t o = rank1_dev(rt, tree, offset);
    const uint64_t oe = rank1_dev(rt, tree, offset + size) - o;
    paths[c * L + l] = make_ulonglong2(offset, o);
    if ((c >> (L - 1 - l)) & 1) {
      offset += size - oe;
      size = oe;
    } else {
      size -= oe;
    }
    offset += n;
  }
}

__global__ void fm_count_kernel(const uint64_t* __restrict__ tree, const uint64_t* __restrict__ rt, uint64_t n,
                                int L, const ulonglong2* __restrict__ paths, const uint64_t* __restrict__ C,
                                uint64_t sigma, const uint8_t* __restrict__ pat, const uint64_t* __restrict__ off,
                                uint64_t npat, uint64_t* __restrict__ out) {
  const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npat) return;
  const uint64_t a = off[p], b = off[p + 1];
  uint64_t sp = 0, ep = n;
  for (uint64_t i = b; i > a && sp < ep; --i) {
    const uint64_t c = pat[i - 1];
    if (c >= sigma) {
      ep = sp;
      break;
    }
    const ulonglong2* pc = paths + c * (uint64_t)L;
    uint64_t x = sp, y = ep;
    for (int l = 0; l < L; ++l) {
      const ulonglong2 nd = __ldg(pc + l);
      const uint64_t rx = rank1_dev(rt, tree, nd.x + x) - nd.y;
      const uint64_t ry = rank1_dev(rt, tree, nd.x + y) - nd.y;
      const bool one = (c >> (L - 1 - l)) & 1;
      x = one ? rx : x - rx;
      y = one ? ry : y - ry;
    }
    const uint64_t base = __ldg(C + c);
    sp = base + x;
    ep = base + y;
  }
  out[p] = ep > sp ? ep - sp : 0;
}

}  // namespace

int launch_fm_count(TreeImpl& t, const uint64_t* C, uint64_t sigma, const uint8_t* pat, const uint64_t* off,
                    uint64_t npat, uint64_t* out, cudaStream_t s) {
  int rc;
  if (!(t.flags & WTG_RANK)) return fail(WTG_ERR_INVALID, "tree built without rank support");
  if (sigma == 0 || sigma > 256 || (t.levels < 63 && sigma > (1ull << t.levels)))
    return fail(WTG_ERR_INVALID, "sigma must be 1..256 and at most 2^levels");
  if (npat == 0) return WTG_OK;
  if ((rc = t.fm_paths.ensure(sigma * t.levels * sizeof(ulonglong2), s))) return rc;
  ulonglong2* paths = t.fm_paths.as<ulonglong2>();
  const uint64_t* tree = t.bits.as<uint64_t>();
  const uint64_t* rt = t.bv.rank.as<uint64_t>();
  count_launch();
  fm_paths_kernel<<<(unsigned)((sigma + 127) / 128), 128, 0, s>>>(tree, rt, t.n, t.levels, sigma, paths);
  WTG_CK(cudaGetLastError());
  count_launch();
  fm_count_kernel<<<(unsigned)((npat + 255) / 256), 256, 0, s>>>(tree, rt, t.n, t.levels, paths, C, sigma, pat,
                                                                 off, npat, out);
  WTG_CK(cudaGetLastError());
  return WTG_OK;
}

}  // namespace wtg
