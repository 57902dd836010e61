// Exact-C9 ATM term of the plain FP64 method (D4ATMExact:
// dispersion/threebody.py:276-302 with RadiiBJMixin 241-256 and
// get_atm_dispersion 54-163; the method class DispD4Exact,
// dispersion/d4.py:67-84):
//
//   C9_ijk = (3/pi) sum_w w_w a_i(w) a_j(w) a_k(w)
//
// with a_i the weighted polarisabilities at q = 0 (the ATM term is not
// charge dependent).  D4: a_i = A0_i (model/d4.py:291-307).  D4S:
// get_weighted_pols (model/d4s.py:292-316) sums the pair-weighted
// polarisabilities over the partner index and divides by the number of real
// atoms, so every atom of element e gets the same vector
// abar_e = (1/nat) sum_n A0_n^(e), where A0_n^(e) is atom n's polarisability
// weighted for partner element e -- one 23-vector per structure and slot.
//
// The triple geometry, damping, cutoff mask and per-atom attribution are the
// ones of the approximate-C9 kernel; only C9 and its adjoint differ.  The
// adjoint of C9 needs dE/da for all three atoms of a triple, so instead of
// pair accumulators the kernel gives each atom x a warp that visits every
// triple containing x once (pairs {y < z} without x): the warp sums x's
// energy share, the ATM force on x and dE/da_x(w) without atomics.  Every
// triple is evaluated three times (once per atom); this term is not on the
// default dftd4() path.
#include "d4_common.cuh"
#include "d4_kernels.cuh"

namespace d4 {

// a_i(w) of every atom (zero for padding): D4 copies A0, D4S writes the
// slot averages.  CTA per structure; S * 23 doubles of shared memory.
__global__ void __launch_bounds__(256) exact_alpha_kernel(Ctx c) {
  extern __shared__ double s_abar[];  // [S][23], D4S only
  __shared__ int s_nat;
  const int b = blockIdx.x;
  const int N = c.N, S = c.S;
  const int n = c.w.n_eff[b];
  const int *Zb = c.w.z + (size_t)b * N;
  const bool d4s = c.cfg.kind == D4_MODEL_D4S;
  if (d4s) {
    if (threadIdx.x == 0) s_nat = 0;
    __syncthreads();
    int cnt = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) cnt += Zb[i] != 0;
    atomicAdd(&s_nat, cnt);
    __syncthreads();
    const double inv = s_nat > 0 ? 1.0 / (double)s_nat : 0.0;
    const int nsl = c.w.n_slots[b];
    for (int t = threadIdx.x; t < S * NFREQ; t += blockDim.x) {
      const int s = t / NFREQ, w = t % NFREQ;
      double acc = 0.0;
      if (s < nsl)
        for (int m = 0; m < n; ++m) {
          const size_t a = (size_t)b * N + m;
          if (Zb[m] != 0) acc += c.w.A0[(a * S + s) * NFREQ + w];
        }
      s_abar[t] = acc * inv;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < N * NFREQ; t += blockDim.x) {
    const int i = t / NFREQ, w = t % NFREQ;
    const size_t a = (size_t)b * N + i;
    double v = 0.0;
    if (i < n && Zb[i] != 0)
      v = d4s ? s_abar[c.w.slot[a] * NFREQ + w] : c.w.A0[a * NFREQ + w];  // D4: S = 1
    c.w.ax[a * NFREQ + w] = v;
  }
}

// Warp per atom x, loop over y (uniform), lanes over z > y.  Pair records
// (r, 1/r, log(R0/r)) come from the pair kernel.
template <bool GRAD, bool PGRAD>
__global__ void __launch_bounds__(256) atm_exact_kernel(Ctx c) {
  __shared__ double s_u[8][NFREQ];  // (3/pi) w_w a_x(w) a_y(w) for the current y
  __shared__ double s_v[8][NFREQ];  // (3/pi) w_w a_y(w)
  const int b = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x = blockIdx.x * 8 + warp;
  const int N = c.N;
  if (x >= N) return;  // whole warp; the kernel has no CTA barrier
  const size_t axx = (size_t)b * N + x;
  const int n = c.w.n_eff[b];
  const int *Zb = c.w.z + (size_t)b * N;
  if (x >= n || Zb[x] == 0) {
    if (lane == 0) c.w.e3[axx] = 0.0;
    if (GRAD) {
      if (lane < 3) c.w.f3x[3 * axx + lane] = 0.0;
      if (lane < NFREQ) c.w.gax[axx * NFREQ + lane] = 0.0;
    }
    return;
  }
  const double cut = c.par.cut_disp3;
  const double alp3 = c.par.alp / 3.0;
  const double s9 = c.par.s9;
  const size_t base = (size_t)b * N * N;
  const double *P = c.positions + (size_t)b * N * 3;
  const double px = P[3 * x], py = P[3 * x + 1], pz = P[3 * x + 2];
  const double wx = atom_weight(c, axx);
  const double *AX = c.w.ax + (size_t)b * N * NFREQ;
  const double cw = lane < NFREQ ? THOPI * c.tab.freq_weights[lane] : 0.0;
  const double ax_l = lane < NFREQ ? AX[(size_t)x * NFREQ + lane] : 0.0;
  double Ex = 0.0, fx = 0.0, fy = 0.0, fz = 0.0, dax = 0.0;
  double g_s9 = 0.0, g_alp = 0.0, g_a1 = 0.0, g_a2 = 0.0;
  for (int y = 0; y < n; ++y) {
    if (y == x || Zb[y] == 0) continue;  // warp-uniform
    const size_t oxy = base + (size_t)x * N + y;
    const double rxy = c.w.pr_r[oxy], irxy = c.w.pr_ir[oxy], Lxy = c.w.pr_L[oxy];
    const bool mxy = rxy <= cut;
    const double wy = atom_weight(c, (size_t)b * N + y);
    const double qx = px - P[3 * y], qy = py - P[3 * y + 1], qz = pz - P[3 * y + 2];
    __syncwarp();
    if (lane < NFREQ) {
      const double ay = AX[(size_t)y * NFREQ + lane];
      s_v[warp][lane] = cw * ay;
      s_u[warp][lane] = cw * ay * ax_l;
    }
    __syncwarp();
    double T[NFREQ];
    if (GRAD) {
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) T[w] = 0.0;
    }
    for (int z = y + 1 + lane; z < n; z += 32) {
      if (z == x || Zb[z] == 0) continue;
      const size_t oxz = base + (size_t)x * N + z, oyz = base + (size_t)y * N + z;
      const double rxz = c.w.pr_r[oxz], ryz = c.w.pr_r[oyz];
      const bool mxz = rxz <= cut, myz = ryz <= cut;
      // shares of the ordered triples (reference mask tests r_ij and r_jk)
      const double mi = (double)(myz * (mxy + mxz));
      const double mj = (double)(mxz * (mxy + myz));
      const double mk = (double)(mxy * (mxz + myz));
      if (mi + mj + mk == 0.0) continue;
      const double *az = AX + (size_t)z * NFREQ;
      double c9 = 0.0;
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) c9 += s_u[warp][w] * az[w];
      const double irxz = c.w.pr_ir[oxz], iryz = c.w.pr_ir[oyz];
      const double X = rxy * rxy, Y = rxz * rxz, Zs = ryz * ryz;
      const double ir1 = irxy * irxz * iryz;
      const double ir2 = ir1 * ir1;
      const double ir3 = ir1 * ir2;
      const double A = X + Zs - Y, Bv = X - Zs + Y, Cv = -X + Zs + Y;
      const double ang = ir3 * (0.375 * A * Bv * Cv * ir2 + 1.0);
      const double Lsum = Lxy + c.w.pr_L[oxz] + c.w.pr_L[oyz];
      const double ta = exp(alp3 * Lsum);
      const double fd = 1.0 / (1.0 + 6.0 * ta);
      const double e = s9 * c9 * fd * ang;
      Ex += e * (1.0 / 6.0) * mi;
      if (GRAD) {
        const double wz = atom_weight(c, (size_t)b * N + z);
        const double wgt = (wx * mi + wy * mj + wz * mk) * (1.0 / 6.0);
        const double K = s9 * c9;
        const double dfl = 6.0 * alp3 * ta * fd * fd;
        const double Q = -(5.0 * ang - 2.0 * ir3);
        const double U = K * fd * 0.375 * ir2 * ir3;
        const double V = 0.5 * K * (fd * Q + ang * dfl);
        const double BC = Bv * Cv, AC = A * Cv, AB = A * Bv;
        const double dex = U * (BC + AC - AB) + V * irxy * irxy;  // d e / d r_xy^2
        const double dey = U * (-BC + AC + AB) + V * irxz * irxz;  // d e / d r_xz^2
        const double rx = px - P[3 * z], ry = py - P[3 * z + 1], rz = pz - P[3 * z + 2];
        fx += 2.0 * wgt * (dex * qx + dey * rx);
        fy += 2.0 * wgt * (dex * qy + dey * ry);
        fz += 2.0 * wgt * (dex * qz + dey * rz);
        const double gc9 = wgt * s9 * fd * ang;  // d(weighted energy) / d C9
#pragma unroll
        for (int w = 0; w < NFREQ; ++w) T[w] += gc9 * az[w];
        if (PGRAD && x < y) {  // x < y < z: each triple once
          const double dfdL = -6.0 * fd * fd * ta;
          g_s9 += wgt * c9 * fd * ang;
          g_alp += wgt * s9 * c9 * ang * dfdL * Lsum * (1.0 / 3.0);
          const double dfa = wgt * s9 * c9 * ang * dfdL * alp3;
          g_a1 += dfa * (c.w.pr_da1[oxy] + c.w.pr_da1[oxz] + c.w.pr_da1[oyz]);
          g_a2 += dfa * (c.w.pr_da2[oxy] + c.w.pr_da2[oxz] + c.w.pr_da2[oyz]);
        }
      }
    }
    if (GRAD) {
      // dE/da_x(w) += (3/pi) w_w a_y(w) sum_z gc9 a_z(w)
#pragma unroll
      for (int w = 0; w < NFREQ; ++w) {
        const double t = warp_sum(T[w]);
        if (lane == w) dax += s_v[warp][w] * t;
      }
    }
  }
  Ex = warp_sum(Ex);
  if (lane == 0) c.w.e3[axx] = Ex;
  if (GRAD) {
    fx = warp_sum(fx);
    fy = warp_sum(fy);
    fz = warp_sum(fz);
    if (lane == 0) {
      c.w.f3x[3 * axx] = fx;
      c.w.f3x[3 * axx + 1] = fy;
      c.w.f3x[3 * axx + 2] = fz;
    }
    if (lane < NFREQ) c.w.gax[axx * NFREQ + lane] = dax;
  }
  if (PGRAD) {
    g_s9 = warp_sum(g_s9);
    g_alp = warp_sum(g_alp);
    g_a1 = warp_sum(g_a1);
    g_a2 = warp_sum(g_a2);
    if (lane == 0) {
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 3], g_a1);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 4], g_a2);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 5], g_s9);
      atomicAdd(&c.w.pgrad[b * D4_PARAM_GRAD_STRIDE + 6], g_alp);
    }
  }
}

// D4S: gbar_s(w) = (1/nat) sum over the atoms m of slot s of dE/da_m(w),
// the adjoint of every atom's slot-s polarisability A0_n^(s).  CTA per
// structure.
__global__ void __launch_bounds__(256) exact_fold_kernel(Ctx c) {
  __shared__ int s_nat;
  const int b = blockIdx.x;
  const int N = c.N, S = c.S;
  const int n = c.w.n_eff[b];
  const int *Zb = c.w.z + (size_t)b * N;
  if (threadIdx.x == 0) s_nat = 0;
  __syncthreads();
  int cnt = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) cnt += Zb[i] != 0;
  atomicAdd(&s_nat, cnt);
  __syncthreads();
  const double inv = s_nat > 0 ? 1.0 / (double)s_nat : 0.0;
  for (int t = threadIdx.x; t < S * NFREQ; t += blockDim.x) {
    const int s = t / NFREQ, w = t % NFREQ;
    double acc = 0.0;
    for (int m = 0; m < n; ++m) {
      const size_t a = (size_t)b * N + m;
      if (Zb[m] != 0 && c.w.slot[a] == s) acc += c.w.gax[a * NFREQ + w];
    }
    c.w.gbar[((size_t)b * S + s) * NFREQ + w] = acc * inv;
  }
}

void launch_atm_exact(const Ctx &c, cudaStream_t st) {
  const bool grad = (c.flags & D4_FLAG_GRADIENT) != 0;
  const bool pgrad = (c.flags & D4_FLAG_PARAM_GRAD) != 0;
  const size_t smem = c.cfg.kind == D4_MODEL_D4S ? (size_t)8 * c.S * NFREQ : 0;
  exact_alpha_kernel<<<c.B, 256, smem, st>>>(c);
  const dim3 atoms((c.N + 7) / 8, c.B);
  if (pgrad)
    atm_exact_kernel<true, true><<<atoms, 256, 0, st>>>(c);
  else if (grad)
    atm_exact_kernel<true, false><<<atoms, 256, 0, st>>>(c);
  else
    atm_exact_kernel<false, false><<<atoms, 256, 0, st>>>(c);
  if (grad && c.cfg.kind == D4_MODEL_D4S) exact_fold_kernel<<<c.B, 256, 0, st>>>(c);
}

}  // namespace d4
