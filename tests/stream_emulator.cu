// CPU check of the triangular-solve streams (test infrastructure only).
//
// Builds the forward (G) and backward (G^T) streams of a factor with the
// library's own host-side builder (build_dir_streams, host copy, no device),
// then executes them on the CPU in the order the kernels do: per stage the
// external entries, then per piece block after block.  Warp format: every
// column a row reads must be solved and still held by the window of solved
// values.  Pipeline format: the kernel's schedule -- in step s the gatherers
// sum block s+2's far entries from columns solved before step s, the reducer
// forms w = T^-1 (acc - far) of block s+1, the mixer y = -Q x of block s+1
// from block s-1, the solver retires block s as w + y - P x of block s-1.  32-wide (k-team) format:
// helpers one block ahead, the solver with the previous block.  A record that
// reads a column not solved at that point would race on the GPU and fails
// the check; the results are compared with plain substitution on the CSR of G.
//
//   stream_emulator <dir> <format 0=warp|1=by stage|2=pipeline> <precision 0=FP64|1=FP32> <kwidth 1|32> [infer]
//
// <dir> holds hdr.bin (n, nnz, len(result_idx)), rp.bin / ci.bin / v.bin (CSR
// of G^T: int64, int32, f64) and ridx.bin (result_idx, int64); with "infer"
// the tree is read off G's pattern instead (tree_infer.hpp).  Prints one
// line "ok rel_fwd rel_bwd team_pieces steps warp_pieces" or "FAIL ..." (exit code 1).

#include "../rchol_gb300/csrc/trsv.cu"
#include "../rchol_gb300/csrc/tree_infer.hpp"

#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <string>

namespace rchol {
// the few library functions trsv.cu calls that live in other files
int host_threads() { return 1; }
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)> &body, int64_t) { body(0, n); }
void note_launch(int64_t) {}
void set_last_error(const std::string &) {}
}  // namespace rchol

using namespace rchol;

namespace {

template <typename T>
std::vector<T> read_file(const std::string &path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(T)));
  if (!f) {
    std::printf("FAIL cannot read %s\n", path.c_str());
    std::exit(1);
  }
  return v;
}

[[noreturn]] void fail(const char *what, long a, long b) {
  std::printf("FAIL %s %ld %ld\n", what, a, b);
  std::exit(1);
}

template <typename VT>
VT ld(const unsigned char *p, size_t idx) {
  VT x;
  std::memcpy(&x, p + sizeof(VT) * idx, sizeof(VT));
  return x;
}

uint32_t col_at(const unsigned char *p, size_t idx, uint32_t csz) {
  if (csz == 2) {
    uint16_t c;
    std::memcpy(&c, p + 2 * idx, 2);
    return c;
  }
  uint32_t c;
  std::memcpy(&c, p + 4 * idx, 4);
  return c;
}

// x = T^-1 t with the packed inverse of a record
template <typename VT>
void apply_inverse(const unsigned char *minv, const VT *t, VT *x, bool upper) {
  for (int r = 0; r < BS; ++r) {
    VT s = 0;
    for (int c = 0; c < BS; ++c) {
      const bool in = upper ? (r <= c) : (r >= c);
      if (in) s += ld<VT>(minv, (size_t)tri_col_off(c, upper) + (size_t)(upper ? r : r - c)) * t[c];
    }
    x[r] = s;
  }
}

// x = T^-1 t with the row-quad packed inverse of a warp- or pipeline-format record
template <typename VT>
void apply_tinv(const unsigned char *tinv, const VT *t, VT *x, bool upper) {
  for (int r = 0; r < BS; ++r) {
    VT s = 0;
    for (int q = tq_lo(r, upper); q <= tq_hi(r, upper); ++q)
      for (int j = 0; j < 4; ++j) {
        const int c = 4 * q + j;
        const VT m = ld<VT>(tinv, 4 * (size_t)(tq_off(r, upper) + q - tq_lo(r, upper)) + j);
        if ((upper ? c < r : c > r) && m != (VT)0) fail("inverse entry outside the triangle", r, c);
        s += m * t[c];
      }
    x[r] = s;
  }
}

template <typename VT>
std::vector<double> emulate(const HostStreamCopy &H, const std::vector<double> &rhs, int64_t n, bool upper,
                            long &team_pieces, long &warp_pieces) {
  std::vector<double> out(n, 0.0);
  std::vector<char> done(n, 0);
  const uint32_t vsz = sizeof(VT);
  for (size_t st = 0; st + 1 < H.stage_ptr.size(); ++st) {
    std::vector<VT> acc(n, 0);
    // external entries: columns outside the piece, all solved in earlier stages
    for (int k = H.stage_ptr[st]; k < H.stage_ptr[st + 1]; ++k) {
      const NodeDesc &nd = H.desc[k];
      for (int r = 0; r < nd.rows; ++r) {
        const int64_t i = nd.begin + r;
        VT s = 0;
        for (int64_t q = H.ext_rp[i]; q < H.ext_rp[i + 1]; ++q) {
          const int64_t c = H.ext_ci[q];
          if (c < 0 || c >= n || !done[c]) fail("external column not yet solved", (long)c, (long)st);
          s += (VT)H.ext_v[q] * (VT)out[c];
        }
        acc[i] = (VT)rhs[i] - s;
      }
    }
    const int fmt = H.stage_fmt[st];
    for (int k = H.stage_ptr[st]; k < H.stage_ptr[st + 1]; ++k) {
      const NodeDesc &nd = H.desc[k];
      std::vector<VT> xs(nd.rows);
      std::vector<int> solved_at(nd.rows, -1);  // block step that solved a piece row
      for (int r = 0; r < nd.rows; ++r) xs[r] = acc[nd.begin + r];
      auto rec = [&](int b) {
        const int64_t o = H.blk_off[nd.blk0 + b];
        if (o < 0 || o >= (int64_t)H.blocks.size() || (o & 15)) fail("record offset", (long)o, b);
        return H.blocks.data() + o;
      };
      auto rec_len = [&](int b) { return H.blk_off[nd.blk0 + b + 1] - H.blk_off[nd.blk0 + b]; };
      auto finish = [&](int b, uint32_t nr, uint32_t row0, const VT *x) {
        if (row0 + nr > (uint32_t)nd.rows) fail("block rows outside the piece", row0, b);
        for (uint32_t r = 0; r < nr; ++r) {
          if (solved_at[row0 + r] >= 0) fail("row solved twice", row0 + r, b);
          xs[row0 + r] = x[r];
          solved_at[row0 + r] = b;
        }
      };
      if (fmt == FMT_WARP) {
        // the window of solved values: slot i % W holds the row written last
        const int64_t W = H.stage_window[st];
        if (W < 64 || (W & (W - 1))) fail("window size", (long)W, k);
        std::vector<int64_t> slot(W, -1);
        ++warp_pieces;
        for (int b = 0; b < nd.nblocks; ++b) {
          const unsigned char *p = rec(b);
          uint32_t hdr[4];
          std::memcpy(hdr, p, 16);
          const uint32_t nr = hdr[0], row0 = hdr[1], nent = hdr[2], csz = hdr[3];
          const W2Layout L = w2_layout(nent, csz, vsz);
          if ((int64_t)L.len != rec_len(b)) fail("warp record length", (long)L.len, b);
          if ((int)L.len > nd.maxrec) fail("record above the piece's maximum", (long)L.len, nd.maxrec);
          uint16_t off[BS + 1];
          std::memcpy(off, p + L.o_eoff, sizeof(off));
          if (off[BS] != nent) fail("warp entry offsets", off[BS], nent);
          VT t[BS] = {}, x[BS];
          for (uint32_t r = 0; r < nr; ++r) {
            VT s0 = 0, s1 = 0;
            for (uint32_t e = off[r]; e < off[r + 1]; ++e) {
              const uint32_t c = col_at(p + L.o_col, e, csz);
              if (c >= (uint32_t)nd.rows || solved_at[c] < 0) fail("warp-format column not yet solved", c, b);
              if (slot[c & (W - 1)] != (int64_t)c) fail("warp-format column no longer in the window", c, b);
              ((e - off[r]) & 1 ? s1 : s0) += ld<VT>(p + L.o_val, e) * xs[c];
            }
            t[r] = xs[row0 + r] - (s0 + s1);
          }
          apply_tinv<VT>(p + L.o_tinv, t, x, upper);
          finish(b, nr, row0, x);
          for (uint32_t r = 0; r < nr; ++r) slot[(row0 + r) & (W - 1)] = row0 + r;
        }
      } else if (fmt == FMT_PIPE) {
        ++team_pieces;
        // the kernel's schedule: in step s the gatherers sum block s+2's far
        // entries, the reducer forms w = T^-1 (acc - far) of block s+1, the
        // mixer y = -Q x of block s+1 from block s-1, the solver retires block
        // s as w + y - P x of block s-1
        const int nb = nd.nblocks;
        std::vector<std::vector<VT>> part(2);
        std::vector<VT> wv(2 * BS, (VT)NAN), yv(2 * BS, (VT)NAN);
        auto hdr_of = [&](int b, uint32_t h[16]) {
          const unsigned char *p = rec(b);
          std::memcpy(h, p, 64);
          const PipeLayout L = pipe_layout(h[4], h[5], h[6], vsz);
          if ((int64_t)L.len != rec_len(b)) fail("pipeline record length", (long)L.len, b);
          if ((int)L.len > nd.maxrec) fail("record above the piece's maximum", (long)L.len, nd.maxrec);
          if (h[7] != L.o_crow || h[8] != L.o_fc || h[9] != L.o_fv || h[10] != (uint32_t)pq_stride(vsz))
            fail("pipeline record offsets", b, 0);
          if ((int)h[4] > nd.maxchunk) fail("chunks above the piece's maximum", h[4], nd.maxchunk);
          return p;
        };
        // dense 32x32 matrix (row stride `stride`) times the 32 unknowns of a
        // block solved in step `when`; every nonzero column must be such an unknown
        auto dense_mul = [&](const unsigned char *M, int r, uint32_t base, int when, int b, const char *what) {
          const int stride = pq_stride(vsz);
          VT acc = 0;
          for (int c = 0; c < BS; ++c) {
            const VT m = ld<VT>(M, (size_t)r * stride + c);
            if (m == (VT)0) continue;
            if (base + c >= (uint32_t)nd.rows || solved_at[base + c] != when) fail(what, c, b);
            acc += m * xs[base + c];
          }
          return acc;
        };
        for (int s = -2; s < nb; ++s) {
          std::vector<VT> newpart;
          if (s + 2 < nb) {  // gatherers
            uint32_t h[16];
            const unsigned char *p = hdr_of(s + 2, h);
            const uint32_t nchunk = h[4], clen = h[5], csz = h[6];
            newpart.assign(nchunk, 0);
            for (uint32_t c = 0; c < nchunk; ++c) {
              VT s0 = 0, s1 = 0;
              for (uint32_t j = 0; j < clen; ++j) {
                const size_t at = (size_t)j * nchunk + c;
                const uint32_t col = col_at(p + h[8], at, csz);
                const VT val = ld<VT>(p + h[9], at);
                if (col >= (uint32_t)nd.rows) fail("far column outside the piece", col, s + 2);
                if (val != (VT)0 && (solved_at[col] < 0 || solved_at[col] > s - 1))
                  fail("far column not solved before the step", col, s + 2);
                (j & 1 ? s1 : s0) += val * xs[col];
              }
              newpart[c] = s0 + s1;
            }
          }
          std::vector<VT> neww, newy;
          if (s + 1 >= 0 && s + 1 < nb) {  // reducer and mixer
            const int bk = s + 1;
            uint32_t h[16];
            const unsigned char *p = hdr_of(bk, h);
            const uint32_t nr = h[0], row0 = h[1], pprow0 = h[3];
            uint16_t crow[BS + 1];
            std::memcpy(crow, p + h[7], sizeof(crow));
            if (crow[BS] != h[4]) fail("chunk rows", crow[BS], h[4]);
            const std::vector<VT> &pb = part[bk & 1];
            if (pb.size() != h[4]) fail("chunk sums not prepared", bk, (long)pb.size());
            VT t[BS] = {};
            for (uint32_t r = 0; r < nr; ++r) {
              if (solved_at[row0 + r] >= 0) fail("reducer row already solved", row0 + r, bk);
              VT f0 = 0, f1 = 0;
              for (uint32_t c = crow[r]; c < crow[r + 1]; ++c) ((c - crow[r]) & 1 ? f1 : f0) -= pb[c];
              t[r] = xs[row0 + r] + (f0 + f1);
            }
            neww.assign(BS, 0);
            apply_tinv<VT>(p + 64, t, neww.data(), upper);
            newy.assign(BS, 0);
            const PipeLayout L = pipe_layout(h[4], h[5], h[6], vsz);
            for (int r = 0; r < BS; ++r)
              newy[r] = bk >= 2 ? -dense_mul(p + L.o_q, r, pprow0, s - 1, bk, "distance-2 column not in block k-2")
                                : (VT)0;
          }
          if (s >= 0) {  // solver
            uint32_t h[16];
            const unsigned char *p = hdr_of(s, h);
            const uint32_t nr = h[0], row0 = h[1], prow0 = h[2];
            const PipeLayout L = pipe_layout(h[4], h[5], h[6], vsz);
            VT x[BS];
            for (int r = 0; r < BS; ++r) {
              if (std::isnan((double)wv[(s & 1) * BS + r]) || std::isnan((double)yv[(s & 1) * BS + r]))
                fail("w or y not prepared", r, s);
              const VT px = s >= 1 ? dense_mul(p + L.o_p, r, prow0, s - 1, s, "distance-1 column not in block k-1")
                                   : (VT)0;
              x[r] = (wv[(s & 1) * BS + r] + yv[(s & 1) * BS + r]) - px;
            }
            finish(s, nr, row0, x);
          }
          if (s + 2 < nb) part[(s + 2) & 1] = newpart;
          if (s + 1 >= 0 && s + 1 < nb)
            for (int r = 0; r < BS; ++r) {
              wv[((s + 1) & 1) * BS + r] = neww[r];
              yv[((s + 1) & 1) * BS + r] = newy[r];
            }
        }
      } else {
        ++team_pieces;
        std::vector<VT> u(2 * BS, (VT)NAN);  // u of blocks by parity, as the helpers leave it
        VT xprev[BS] = {};
        for (int b = 0; b < nd.nblocks; ++b) {
          if (b + 1 < nd.nblocks) {  // helpers: far sums of block b+1 (columns solved before block b)
            const unsigned char *p = rec(b + 1);
            uint32_t h[16];
            std::memcpy(h, p, 64);
            const uint32_t nr1 = h[0], row01 = h[1], nchunk = h[4], clen = h[5], csz = h[6];
            const TeamLayout L = team_layout(h[3], h[7], nchunk, clen, csz, vsz);
            if ((int64_t)L.len != rec_len(b + 1)) fail("team record length", (long)L.len, b + 1);
            if (h[11] != L.o_fcol || h[12] != L.o_fval || h[13] != L.o_min) fail("team record offsets", b + 1, 0);
            if ((int)nchunk > nd.maxchunk) fail("chunks above the piece's maximum", nchunk, nd.maxchunk);
            std::vector<VT> part(nchunk);
            for (uint32_t c = 0; c < nchunk; ++c) {
              VT s0 = 0, s1 = 0;
              for (uint32_t j = 0; j < clen; ++j) {
                const size_t at = (size_t)j * nchunk + c;
                const uint32_t col = col_at(p + L.o_fcol, at, csz);
                const VT val = ld<VT>(p + L.o_fval, at);
                if (col >= (uint32_t)nd.rows) fail("far column outside the piece", col, b + 1);
                if (val != (VT)0 && (solved_at[col] < 0 || solved_at[col] > b - 1))
                  fail("far column not solved before the step", col, b + 1);
                (j & 1 ? s1 : s0) += val * xs[col];
              }
              part[c] = s0 + s1;
            }
            uint16_t crow[BS + 1];
            std::memcpy(crow, p + L.o_crow, sizeof(crow));
            if (crow[BS] != nchunk) fail("chunk rows", crow[BS], nchunk);
            for (uint32_t r = 0; r < (uint32_t)BS; ++r) {
              VT f0 = 0, f1 = 0;
              for (uint32_t c = crow[r]; c < crow[r + 1]; ++c) ((c - crow[r]) & 1 ? f1 : f0) += part[c];
              u[((b + 1) & 1) * BS + r] = r < nr1 ? xs[row01 + r] - (f0 + f1) : (VT)0;
            }
          }
          // solver: block b, near entries from block b-1 (slot-major)
          const unsigned char *p = rec(b);
          uint32_t h[16];
          std::memcpy(h, p, 64);
          const uint32_t nr = h[0], row0 = h[1], prow0 = h[2], nmax = h[7];
          const TeamLayout L = team_layout(h[3], nmax, h[4], h[5], h[6], vsz);
          VT t[BS] = {}, x[BS];
          for (uint32_t r = 0; r < nr; ++r) {
            const VT ur = b == 0 ? xs[row0 + r] : u[(b & 1) * BS + r];
            if (std::isnan((double)ur)) fail("u not prepared", r, b);
            VT s0 = 0, s1 = 0;
            for (uint32_t j = 0; j < nmax; ++j) {
              const size_t at = (size_t)j * BS + r;
              const uint32_t c = p[L.o_ncol + at];
              const VT val = ld<VT>(p + L.o_nval, at);
              if (c >= (uint32_t)BS) fail("near column", c, b);
              if (val != (VT)0 && (b == 0 || solved_at[prow0 + c] != b - 1)) fail("near column not in the previous block", c, b);
              (j & 1 ? s1 : s0) += val * xprev[c];
            }
            t[r] = ur - (s0 + s1);
          }
          apply_inverse<VT>(p + L.o_min, t, x, upper);
          for (int r = 0; r < BS; ++r) xprev[r] = r < (int)nr ? x[r] : (VT)0;
          finish(b, nr, row0, x);
        }
      }
      for (int r = 0; r < nd.rows; ++r) {
        if (solved_at[r] < 0) fail("piece row never solved", r, k);
        out[nd.begin + r] = (double)xs[r];
        done[nd.begin + r] = 1;
      }
    }
  }
  for (int64_t i = 0; i < n; ++i)
    if (!done[i]) fail("row outside every piece", (long)i, 0);
  return out;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 5) {
    std::printf("FAIL usage: stream_emulator <dir> <format> <precision> <kwidth>\n");
    return 1;
  }
  const std::string dir = argv[1];
  const int team_mode = std::atoi(argv[2]);
  const bool fp32 = std::atoi(argv[3]) != 0;
  const int kwidth = std::atoi(argv[4]);
  const auto hdr = read_file<int64_t>(dir + "/hdr.bin", 3);
  const int64_t n = hdr[0], nnz = hdr[1], nr = hdr[2];
  const auto rp = read_file<int64_t>(dir + "/rp.bin", n + 1);
  const auto ci = read_file<int32_t>(dir + "/ci.bin", nnz);
  const auto v = read_file<double>(dir + "/v.bin", nnz);
  const auto ri = read_file<int64_t>(dir + "/ridx.bin", nr);
  // tree from result_idx: left half, right half, then the separator
  // (rchol_lap.cpp:187-355)
  std::vector<TreeNode> nodes;
  std::function<void(int64_t, int64_t, int)> split = [&](int64_t start, int64_t total, int depth) {
    if (total == 1) {
      nodes.push_back({ri[start], std::min(ri[start + 1], n), depth, true});
      return;
    }
    const int64_t half = (total - 1) / 2;
    split(start, half, depth + 1);
    split(start + half, half, depth + 1);
    nodes.push_back({ri[start + total - 1], std::min(ri[start + total], n), depth, false});
  };
  split(0, nr - 1, 1);
  // "infer": the tree read off G's pattern (as a factor loaded without one gets)
  const bool infer = argc > 5 && std::string(argv[5]) == "infer";
  if (infer) {
    std::vector<int64_t> ci64(ci.begin(), ci.end());
    nodes = infer_factor_tree(n, rp.data(), ci64.data());
  }
  // G (CSR of rows) = transpose of the CSR of G^T
  std::vector<int64_t> lrp(n + 1, 0);
  for (int32_t c : ci) lrp[c + 1]++;
  for (int64_t i = 0; i < n; ++i) lrp[i + 1] += lrp[i];
  std::vector<int32_t> lci(nnz);
  std::vector<double> lv(nnz);
  std::vector<int64_t> cur(lrp.begin(), lrp.end() - 1);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t q = rp[i]; q < rp[i + 1]; ++q) {
      const int64_t j = ci[q];
      lci[cur[j]] = (int32_t)i;
      lv[cur[j]++] = v[q];
    }
  // substitution references: y = G^-1 b, z = G^-T y
  std::vector<double> b(n), y(n), z(n);
  for (int64_t i = 0; i < n; ++i) b[i] = std::sin(0.37 * (double)i) + 0.1;
  for (int64_t i = 0; i < n; ++i) {
    double s = b[i], d = 0;
    for (int64_t q = lrp[i]; q < lrp[i + 1]; ++q)
      if (lci[q] == i) d = lv[q];
      else s -= lv[q] * y[lci[q]];
    y[i] = s / d;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double s = y[i], d = 0;
    for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
      if (ci[q] == i) d = v[q];
      else s -= v[q] * z[ci[q]];
    z[i] = s / d;
  }
  StreamDir Df, Db;
  HostStreamCopy Hf, Hb;
  build_dir_streams(lrp, lci, lv, n, nodes, false, fp32, team_mode, kwidth, Df, 0, &Hf);
  build_dir_streams(rp, ci, v, n, nodes, true, fp32, team_mode, kwidth, Db, 0, &Hb);
  if (argc > 5 && std::string(argv[5]) == "stats") {  // the plan only: one line per stage
    for (int dir = 0; dir < 2; ++dir) {
      const StreamDir &D = dir ? Db : Df;
      const HostStreamCopy &H = dir ? Hb : Hf;
      std::printf("%s: %zu stages, %lld block steps, %lld record bytes\n", dir ? "backward" : "forward",
                  D.stage_ptr.size() - 1, (long long)D.steps, (long long)H.blocks.size());
      for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
        int64_t rows = 0, blocks = 0, bytes = 0, ext = 0;
        int maxnb = 0;
        for (int k = D.stage_ptr[st]; k < D.stage_ptr[st + 1]; ++k) {
          const NodeDesc &nd = H.desc[k];
          rows += nd.rows;
          blocks += nd.nblocks;
          maxnb = std::max(maxnb, nd.nblocks);
          bytes += H.blk_off[nd.blk0 + nd.nblocks] - H.blk_off[nd.blk0];
          ext += H.ext_rp[nd.begin + nd.rows] - H.ext_rp[nd.begin];
        }
        std::printf("  st %2zu fmt %d pieces %5d rows %9lld maxrows %6d steps %5d maxrec %6d win %5d warps %2d "
                    "chunks %4d recMB %8.1f ext %10lld\n",
                    st, D.stage_fmt[st], D.stage_ptr[st + 1] - D.stage_ptr[st], (long long)rows, D.stage_rows[st],
                    maxnb, D.stage_maxrec[st], D.stage_window[st], D.stage_warps[st], D.stage_chunks[st],
                    bytes / 1e6, (long long)ext);
      }
    }
    return 0;
  }
  long tf = 0, tb = 0, wf = 0, wb = 0;
  const auto ye = fp32 ? emulate<float>(Hf, b, n, false, tf, wf) : emulate<double>(Hf, b, n, false, tf, wf);
  const auto ze = fp32 ? emulate<float>(Hb, y, n, true, tb, wb) : emulate<double>(Hb, y, n, true, tb, wb);
  double ey = 0, ny = 0, ez = 0, nz = 0;
  for (int64_t i = 0; i < n; ++i) {
    ey += (ye[i] - y[i]) * (ye[i] - y[i]);
    ny += y[i] * y[i];
    ez += (ze[i] - z[i]) * (ze[i] - z[i]);
    nz += z[i] * z[i];
  }
  std::printf("ok %.3e %.3e %ld %ld %ld\n", std::sqrt(ey / ny), std::sqrt(ez / nz), tf + tb, (long)(Df.steps + Db.steps),
              wf + wb);
  return 0;
}
