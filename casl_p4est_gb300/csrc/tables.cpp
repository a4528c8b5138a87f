// Flattener: node-neighbour records -> FP64 structure-of-arrays tables (see tables.hpp).
#include "tables.hpp"

#include <stdexcept>

namespace lsg {

template <int D>
void build_tables64(const Forest<D>& F, Tables64<D>& T) {
  constexpr int H = Dim<D>::HALF;
  constexpr int NS = 2 * D * H;
  const int64_t N = (int64_t)F.num_nodes();
  T.N = N;
  T.nbr.assign((size_t)NS * N, -1);
  T.w.assign((size_t)NS * N, 0.0);
  T.nrm.assign((size_t)2 * D * N, 0.0);
  T.d.assign((size_t)2 * D * N, 0.0);
  T.q.assign((size_t)2 * D * (D - 1) * N, 0.0);
  T.cidx.assign((size_t)N, -1);
  T.wall.assign((size_t)N, 0);
  T.smin.assign((size_t)N, 0.0);
  std::vector<uint8_t> needs(N, 0);
  int failed = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : failed)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    const int32_t n = (int32_t)nn;
    Qnnn<D> q;
    if (construct_neighbors<D>(F, n, q)) {
      ++failed;
      continue;
    }
    needs[n] = fill_row64<D>(q, N, n, T.nbr.data(), T.w.data(), T.nrm.data(), T.d.data(), T.q.data(), T.smin.data()) ? 1 : 0;
    T.wall[n] = (uint8_t)wall_mask<D>(F, n);
  }
  if (failed) throw std::runtime_error("node neighbours: incomplete stencil in a single-process forest");
  int32_t R = 0;
  for (int64_t n = 0; n < N; ++n)
    if (needs[n]) T.cidx[n] = R++;
  T.crec.assign((size_t)6 * R, 0.0);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    const int32_t r = T.cidx[nn];
    if (r < 0) continue;
    Qnnn<D> q;
    construct_neighbors<D>(F, (int32_t)nn, q);
    cross_terms<D>(q, &T.crec[(size_t)6 * r]);
  }
}

template <int D>
void build_gradient_tables(const Forest<D>& F, std::vector<int32_t>& gidx, std::vector<double>& grec, std::vector<uint8_t>& gmask) {
  constexpr int W = D * (D - 1);
  const int64_t N = (int64_t)F.num_nodes();
  std::vector<double> wbuf((size_t)W * N);
  std::vector<uint8_t> mbuf((size_t)N, 0);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    Qnnn<D> q;
    construct_neighbors<D>(F, (int32_t)nn, q);
    uint8_t mask = 0;
    for (int a = 0; a < D; ++a)
      for (int j = 0; j < D - 1; ++j) {
        // dd_correction_weight_to_naive_first_derivative(d_m, d_p, d_m_m, d_m_p, d_p_m, d_p_p)
        const double d_m = q.d[2 * a], d_p = q.d[2 * a + 1];
        const double d_m_m = q.dt[2 * a][2 * j], d_m_p = q.dt[2 * a][2 * j + 1];
        const double d_p_m = q.dt[2 * a + 1][2 * j], d_p_p = q.dt[2 * a + 1][2 * j + 1];
        const double w = 0.5 * (d_p_m * d_p_p * d_m / d_p - d_m_m * d_m_p * d_p / d_m) / (d_m + d_p);
        wbuf[(size_t)nn * W + a * (D - 1) + j] = w;
        if (!(fabs(w * q.inverse_d_max) < EPS)) mask |= (uint8_t)(1u << (a * (D - 1) + j));
      }
    mbuf[(size_t)nn] = mask;
  }
  gidx.assign((size_t)N, -1);
  int32_t R = 0;
  for (int64_t n = 0; n < N; ++n)
    if (mbuf[(size_t)n]) gidx[(size_t)n] = R++;
  grec.assign((size_t)W * R, 0.0);
  gmask.assign((size_t)R, 0);
  for (int64_t n = 0; n < N; ++n) {
    const int32_t r = gidx[(size_t)n];
    if (r < 0) continue;
    for (int k = 0; k < W; ++k) grec[(size_t)r * W + k] = wbuf[(size_t)n * W + k];
    gmask[(size_t)r] = mbuf[(size_t)n];
  }
}

template void build_gradient_tables<2>(const Forest<2>&, std::vector<int32_t>&, std::vector<double>&, std::vector<uint8_t>&);
template void build_gradient_tables<3>(const Forest<3>&, std::vector<int32_t>&, std::vector<double>&, std::vector<uint8_t>&);

template <int D>
void build_corner_neighbors(const Forest<D>& F, std::vector<int32_t>& out) {
  constexpr int CH = Dim<D>::CHILDREN;
  constexpr int K = D == 3 ? 12 : 4;
  const int64_t N = (int64_t)F.num_nodes();
  out.assign((size_t)K * N, -1);
#pragma omp parallel for schedule(dynamic, 4096)
  for (long long nn = 0; nn < (long long)N; ++nn) {
    const int32_t n = (int32_t)nn;
    // the 2^D diagonal cells, index bit a set for the + side along a
    int32_t cell[8];
    for (int v = 0; v < CH; ++v) {
      const int c[3] = {(v & 1) ? 1 : -1, (v & 2) ? 1 : -1, (v & 4) ? 1 : -1};
      int32_t quad, tree;
      find_neighbor_cell_of_node<D>(F, n, c, quad, tree);
      cell[v] = quad;
    }
    auto node = [&](int32_t quad, int v) { return F.nd->host().local_nodes[(size_t)quad * CH + v]; };
    auto pick = [&](int c1, int v1, int c2, int v2) -> int32_t {
      return cell[c1] >= 0 ? node(cell[c1], v1) : (cell[c2] >= 0 ? node(cell[c2], v2) : -1);
    };
    int32_t r[12];
    if (D == 2) {
      for (int v = 0; v < 4; ++v) r[v] = cell[v] >= 0 ? node(cell[v], v) : -1;
    } else {
      // cells: mmm=0 pmm=1 mpm=2 ppm=3 mmp=4 pmp=5 mpp=6 ppp=7; corners v = x + 2y + 4z
      r[0] = pick(0, 2, 2, 0);    // m0m
      r[1] = pick(1, 3, 3, 1);    // p0m
      r[2] = pick(4, 6, 6, 4);    // m0p
      r[3] = pick(5, 7, 7, 5);    // p0p
      r[4] = pick(0, 1, 1, 0);    // 0mm
      r[5] = pick(2, 3, 3, 2);    // 0pm
      r[6] = pick(4, 5, 5, 4);    // 0mp
      r[7] = pick(6, 7, 7, 6);    // 0pp
      r[8] = pick(0, 4, 4, 0);    // mm0
      r[9] = pick(1, 5, 5, 1);    // pm0
      r[10] = pick(2, 6, 6, 2);   // mp0
      r[11] = pick(3, 7, 7, 3);   // pp0
    }
    for (int k = 0; k < K; ++k) out[(size_t)k * N + n] = r[k];
  }
}

template void build_corner_neighbors<2>(const Forest<2>&, std::vector<int32_t>&);
template void build_corner_neighbors<3>(const Forest<3>&, std::vector<int32_t>&);

template <int D>
void concat_tables64(const std::vector<const Tables64<D>*>& parts, Tables64<D>& out) {
  constexpr int H = Dim<D>::HALF;
  constexpr int NS = 2 * D * H;
  int64_t N = 0;
  size_t R = 0;
  for (const auto* t : parts) {
    N += t->N;
    R += t->crec.size() / 6;
  }
  out.N = N;
  out.nbr.resize((size_t)NS * N);
  out.w.resize((size_t)NS * N);
  out.nrm.resize((size_t)2 * D * N);
  out.d.resize((size_t)2 * D * N);
  out.q.resize((size_t)2 * D * (D - 1) * N);
  out.cidx.resize((size_t)N);
  out.crec.clear();
  out.crec.reserve(6 * R);
  out.wall.resize((size_t)N);
  out.smin.resize((size_t)N);
  int64_t off = 0;
  int32_t roff = 0;
  for (const auto* t : parts) {
    const int64_t n = t->N;
    for (int sl = 0; sl < NS; ++sl)
      for (int64_t i = 0; i < n; ++i) {
        const int32_t j = t->nbr[(size_t)sl * n + i];
        out.nbr[(size_t)sl * N + off + i] = j >= 0 ? (int32_t)(j + off) : j;
        out.w[(size_t)sl * N + off + i] = t->w[(size_t)sl * n + i];
      }
    for (int dir = 0; dir < 2 * D; ++dir)
      for (int64_t i = 0; i < n; ++i) {
        out.nrm[(size_t)dir * N + off + i] = t->nrm[(size_t)dir * n + i];
        out.d[(size_t)dir * N + off + i] = t->d[(size_t)dir * n + i];
      }
    for (int sl = 0; sl < 2 * D * (D - 1); ++sl)
      for (int64_t i = 0; i < n; ++i) out.q[(size_t)sl * N + off + i] = t->q[(size_t)sl * n + i];
    for (int64_t i = 0; i < n; ++i) {
      const int32_t c = t->cidx[(size_t)i];
      out.cidx[(size_t)(off + i)] = c >= 0 ? c + roff : c;
      out.wall[(size_t)(off + i)] = t->wall[(size_t)i];
      out.smin[(size_t)(off + i)] = t->smin[(size_t)i];
    }
    out.crec.insert(out.crec.end(), t->crec.begin(), t->crec.end());
    off += n;
    roff += (int32_t)(t->crec.size() / 6);
  }
}

template void concat_tables64<2>(const std::vector<const Tables64<2>*>&, Tables64<2>&);
template void concat_tables64<3>(const std::vector<const Tables64<3>*>&, Tables64<3>&);
template void build_tables64<2>(const Forest<2>&, Tables64<2>&);
template void build_tables64<3>(const Forest<3>&, Tables64<3>&);

}  // namespace lsg
