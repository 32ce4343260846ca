// The per-instance full-spectrum eigensolver (isolation, compaction,
// balancing, Hessenberg reduction, repacking and the QR of qr.cuh) run by one
// CTA over a persistent queue.  hqr.cu includes it inside namespace stab,
// after qr.cuh and the phase counters g_eig_phase_cycles; the CPU test of
// the double-word eigensolver compiles it on the host with the CUDA thread
// model replaced by threads of one process.
#pragma once

// dynamic shared memory of eig_plain_body: the active flags and the active
// list (m ints each, rounded up to 16 bytes), then the vectors v, w, z, vn;
// with the QR in shared memory (qr_smem) that region also holds the packed
// Hessenberg matrix of the QR phase
inline size_t eig_plain_smem_bytes(int mmax, bool qr_smem = false) {
  const size_t head = ((2 * (size_t)mmax * sizeof(int) + 15) / 16) * 16;
  size_t vec = 4 * (size_t)mmax;
  if (qr_smem) vec = std::max(vec, (size_t)hess_packed_size(mmax));
  return head + vec * sizeof(zc);
}

// The eigensolver of one CTA over a persistent queue of instances; it runs
// with either block size (HQ_T for the batch, HQ_WIDE for a few instances).
// C is the working precision from the compaction on: complex128, or
// double-word complex.  In double-word form the compacted matrix is scaled
// by a power of two that brings its largest entry near 1 (the float exponent
// range is narrow), again after balancing, and the QR eigenvalues are scaled
// back; the isolated eigenvalues come straight from the FP64 input.
// QS: the QR phase runs on a packed copy of the Hessenberg matrix in shared
// memory (the kernel's dynamic shared memory was sized with qr_smem), the
// other phases on the working matrix in global memory as before.
template <class C, bool QS = false>
__device__ __forceinline__ void eig_plain_body(int count, const int32_t* __restrict__ msz, zc* __restrict__ A,
                                               const int64_t* __restrict__ a_off, zc* __restrict__ Hp,
                                               const int64_t* __restrict__ h_off, zc* __restrict__ eig,
                                               const int64_t* __restrict__ eig_off, int32_t* __restrict__ status,
                                               int32_t* __restrict__ work_counter, const int32_t* __restrict__ order,
                                               double* __restrict__ flops_out, unsigned char* smraw, HqrSmem<C>& s,
                                               int& s_inst) {
  typedef typename ew<C>::real R;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (;;) {
    if (tid == 0) s_inst = atomicAdd(work_counter, 1);
    __syncthreads();
    const int slot = s_inst;
    if (slot >= count) return;
    const int inst = order ? order[slot] : slot;
    const int m = msz[inst];
    zc* M = A + a_off[inst];
    C* Hg = reinterpret_cast<C*>(Hp + h_off[inst]);
    zc* ev = eig + eig_off[inst];
    // shared scratch: active flags and act list (m ints each), then v, w, z
    int* active = reinterpret_cast<int*>(smraw);
    int* act = active + m;
    C* zs = reinterpret_cast<C*>(smraw + ((2 * (size_t)m * sizeof(int) + 15) / 16) * 16);
    C* v = zs;
    C* w = v + m;
    C* z = w + m;
    C* vn = z + m;            // next step's reflector vector (Hessenberg reduction)
    for (int i = tid; i < m; i += NTH) active[i] = 1;
    if (tid == 0) { s.mp = 0; s.emax = 0; }
    __syncthreads();
    long long t_ph = clock64();
    auto phase = [&](int q) {
      if (tid == 0) {
        const long long t = clock64();
        atomicAdd(&g_eig_phase_cycles[q], (unsigned long long)(t - t_ph));
        t_ph = t;
      }
    };
    // ---- 1. isolation -----------------------------------------------------
    int n_iso = 0;           // isolated eigenvalues are written from the top: ev[m-1-q]
    for (int pass = 0; pass < m; ++pass) {
      if (tid == 0) s.found = 0;
      __syncthreads();
      for (int r = tid; r < m; r += NTH) {           // rows: thread per row
        if (!active[r]) continue;
        bool zero = true;
        for (int c = 0; c < m && zero; ++c) {
          if (c == r || !active[c]) continue;
          const zc a = M[(size_t)c * m + r];
          zero = (a.x == 0.0 && a.y == 0.0);
        }
        if (zero) { active[r] = 2; atomicAdd(&s.found, 1); }
      }
      __syncthreads();   // the column test reads the row marks of this pass
      for (int c = warp; c < m; c += NWA) {          // columns: warp per column
        if (active[c] != 1) continue;
        bool zero = true;
        for (int r = lane; r < m; r += 32) {
          if (r == c || active[r] == 0) continue;
          const zc a = M[(size_t)c * m + r];
          if (a.x != 0.0 || a.y != 0.0) zero = false;
        }
        zero = __all_sync(0xffffffffu, zero);
        if (zero && lane == 0) { active[c] = 3; atomicAdd(&s.found, 1); }
      }
      __syncthreads();
      if (s.found == 0) break;
      if (tid == 0) {
        int q = n_iso;
        for (int i = 0; i < m; ++i)
          if (active[i] >= 2) { ev[m - 1 - q] = M[(size_t)i * m + i]; active[i] = 0; ++q; }
        s.kk = q;
      }
      __syncthreads();
      n_iso = s.kk;
      __syncthreads();
    }
    phase(0);
    // ---- 2. compaction ------------------------------------------------------
    if (tid == 0) {
      int q = 0;
      for (int i = 0; i < m; ++i)
        if (active[i]) act[q++] = i;
      s.mp = q;
    }
    __syncthreads();
    const int mp = s.mp;
    const int ld = mp;
    double unscale = 1.0;
    if constexpr (std::is_same<C, zc>::value) {
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) Hg[(size_t)c * ld + r] = M[(size_t)sc * m + act[r]];
      }
    } else {
      // largest binary exponent of the active entries (integer work), then
      // the scaled copy in double-word form
      int emax = 0;
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) {
          const zc a = M[(size_t)sc * m + act[r]];
          emax = max(emax, max((__double2hiint(a.x) >> 20) & 0x7ff, (__double2hiint(a.y) >> 20) & 0x7ff));
        }
      }
      atomicMax(&s.emax, emax);
      __syncthreads();
      // 2^-e with e the unbiased exponent (0 for an all-zero matrix)
      const int e = (s.emax == 0 || s.emax == 0x7ff) ? 0 : s.emax - 1023;
      const double scale = ldexp(1.0, -e);
      unscale = ldexp(1.0, e);
      for (int c = warp; c < mp; c += NWA) {
        const int sc = act[c];
        for (int r = lane; r < mp; r += 32) Hg[(size_t)c * ld + r] = ew<C>::from64(zscale(M[(size_t)sc * m + act[r]], scale));
      }
    }
    __syncthreads();
    phase(1);
    // ---- 3. balancing -------------------------------------------------------
    // (powers of two only, so the norms need little precision: in the
    // double-word form they are taken from the high words in FP32)
    for (int sweep = 0; sweep < 64; ++sweep) {
      if (tid == 0) s.flag = 0;
      __syncthreads();
      for (int i = 0; i < mp; ++i) {
        R cs = 0, rs = 0;
        for (int r = tid; r < mp; r += NTH) {
          if (r == i) continue;
          cs += ew<C>::mag2(Hg[(size_t)i * ld + r]);
          rs += ew<C>::mag2(Hg[(size_t)r * ld + i]);
        }
        block_sum2(s, cs, rs);
        if (tid == 0) {
          R c = sqrt(cs), r = sqrt(rs), f = 1;
          if (c != (R)0 && r != (R)0) {
            R g = r / (R)2;
            const R sum = c + r;
            int guard = 0;
            while (c < g && guard++ < 2000) { f *= (R)2; c *= (R)2; r /= (R)2; g /= (R)2; }
            g = c / (R)2;
            while (g >= r && guard++ < 4000) { f /= (R)2; c /= (R)2; g /= (R)2; r *= (R)2; }
            if (c + r >= (R)0.95 * sum) f = 1;
          }
          s.sc[0] = (double)f;
          if (f != (R)1) s.flag = 1;
        }
        __syncthreads();
        const R f = (R)s.sc[0];
        if (f != (R)1) {
          const R gi = (R)1 / f;
          for (int q = tid; q < mp; q += NTH) {
            C* a = &Hg[(size_t)q * ld + i];    // row i
            *a = zscale(*a, gi);
          }
          __syncthreads();
          for (int q = tid; q < mp; q += NTH) {
            C* a = &Hg[(size_t)i * ld + q];    // column i
            *a = zscale(*a, f);
          }
        }
        __syncthreads();
      }
      if (!s.flag) break;
      __syncthreads();
    }
    if constexpr (!std::is_same<C, zc>::value) {
      // balancing moves the largest entry away from 1: scale again by a power
      // of two (largest float exponent of the high words, integer work)
      if (tid == 0) s.emax = 0;
      __syncthreads();
      int em = 0;
      for (int q = tid; q < mp * mp; q += NTH) {
        const C a = Hg[q];
        em = max(em, max((__float_as_int(a.x) >> 23) & 0xff, (__float_as_int(a.z) >> 23) & 0xff));
      }
      atomicMax(&s.emax, em);
      __syncthreads();
      const int e2 = (s.emax == 0 || s.emax == 0xff) ? 0 : s.emax - 127;
      if (e2 != 0) {
        const float sc2 = ldexpf(1.f, -e2);
        for (int q = tid; q < mp * mp; q += NTH) Hg[q] = zscale(Hg[q], sc2);
        unscale = ldexp(unscale, e2);
      }
      __syncthreads();
    }
    phase(2);
    // ---- 4. Hessenberg reduction -----------------------------------------
    // The left update of step k leaves column k+1 final, so the warp that
    // updates it also copies it into the next step's reflector vector and
    // sums its squared tail: step k+1 starts without a pass or a block
    // reduction of its own.
    double flops = 0.0;   // counted work of the reduction and the sweeps (thread 0)
    bool have_next = false;
    for (int k = 0; k + 2 < mp; ++k) {
      const int L = mp - k - 1;
      if (tid == 0) flops += 16.0 * (double)mp * L + 16.0 * (double)L * L;
      double ss = 0.0;
      if (have_next) {
        C* t = v;                        // the vector gathered by the last step
        v = vn;
        vn = t;
        ss = s.sc[5];
      } else {
        typename ew<C>::sq acc = ew<C>::sq_zero();
        for (int r = tid; r < L; r += NTH) {
          const C x = Hg[(size_t)k * ld + k + 1 + r];
          v[r] = x;
          if (r >= 1) ew<C>::sq_add(acc, x);
        }
        ss = block_sum_sq<C>(s, acc);
      }
      have_next = false;
      if (tid == 0) {
        const zc alpha = ew<C>::to64(v[0]);
        if (ss == 0.0 && alpha.y == 0.0) {
          s.flag = 0;                                      // H(k) = I
        } else {
          s.flag = 1;
          const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + ss), alpha.x);
          const zc scal = zdiv(zmk(1.0, 0.0), zmk(alpha.x - beta, alpha.y));
          s.hc[0] = ew<C>::from64(zmk((beta - alpha.x) / beta, -alpha.y / beta));   // tau
          s.hc[1] = ew<C>::from64(scal);
          s.hc[2] = ew<C>::from64(zmk(beta, 0.0));
        }
      }
      __syncthreads();
      if (!s.flag) continue;
      const C tau = s.hc[0];
      const C scal = s.hc[1];
      for (int r = tid; r < L; r += NTH) v[r] = (r == 0) ? ew<C>::one() : zmul(v[r], scal);
      if (tid == 0) Hg[(size_t)k * ld + k + 1] = s.hc[2];
      for (int r = 2 + tid; r <= L; r += NTH) Hg[(size_t)k * ld + k + r] = ew<C>::zero();
      __syncthreads();
      // right: w = tau H(:, k+1:) v, a row per thread.  Four partial sums
      // over the columns break the dependency chain of the accumulation (the
      // batch runs latency bound, with a third of the issue slots busy).
      for (int r = tid; r < mp; r += NTH) {
        C a0 = ew<C>::zero(), a1 = a0, a2 = a0, a3 = a0;
        const C* row = Hg + (size_t)(k + 1) * ld + r;
        int c = 0;
        for (; c + 4 <= L; c += 4) {
          a0 = zfma(row[(size_t)c * ld], v[c], a0);
          a1 = zfma(row[(size_t)(c + 1) * ld], v[c + 1], a1);
          a2 = zfma(row[(size_t)(c + 2) * ld], v[c + 2], a2);
          a3 = zfma(row[(size_t)(c + 3) * ld], v[c + 3], a3);
        }
        for (; c < L; ++c) a0 = zfma(row[(size_t)c * ld], v[c], a0);
        w[r] = zmul(tau, zadd(zadd(a0, a1), zadd(a2, a3)));
      }
      __syncthreads();
      // right update fused with the left product z = conj(tau) v^H H(k+1:, k+1:),
      // a warp per two columns (two independent chains per lane)
      for (int c = warp; c < L; c += 2 * NWA) {
        const int c2 = c + NWA;
        const bool two = c2 < L;             // uniform over the warp
        const C vc = zconj(v[c]), vc2 = two ? zconj(v[c2]) : ew<C>::zero();
        C* col = Hg + (size_t)(k + 1 + c) * ld;
        C* col2 = Hg + (size_t)(k + 1 + (two ? c2 : c)) * ld;
        C acc = ew<C>::zero(), acc2 = acc;
        for (int r = lane; r < mp; r += 32) {
          const C wr = w[r];
          const C x = col[r], x2 = col2[r];
          const C h = zfnma(wr, vc, x);
          col[r] = h;
          C h2 = x2;
          if (two) {
            h2 = zfnma(wr, vc2, x2);
            col2[r] = h2;
          }
          if (r >= k + 1) {
            const C vr = v[r - k - 1];
            acc = zcfma(vr, h, acc);
            acc2 = zcfma(vr, h2, acc2);
          }
        }
        acc = ew<C>::warp_sum_c(acc);
        acc2 = ew<C>::warp_sum_c(acc2);
        if (lane == 0) {
          z[c] = zmul(zconj(tau), acc);
          if (two) z[c2] = zmul(zconj(tau), acc2);
        }
      }
      __syncthreads();
      // left update: H(k+1:, k+1:) -= v z; column k+1 (c = 0, warp 0) also
      // feeds the next step: vn = H(k+2:, k+1), s.sc[5] = sum |vn[1:]|^2
      for (int c = warp; c < L; c += NWA) {
        const C zc_ = z[c];
        C* col = Hg + (size_t)(k + 1 + c) * ld + k + 1;
        if (c == 0) {
          typename ew<C>::sq sn = ew<C>::sq_zero();
          for (int r = lane; r < L; r += 32) {
            const C h = zfnma(v[r], zc_, col[r]);
            col[r] = h;
            if (r >= 1) vn[r - 1] = h;
            if (r >= 2) ew<C>::sq_add(sn, h);
          }
          sn = warp_sum(sn);
          if (lane == 0) s.sc[5] = ew<C>::sq_64(sn);
        } else {
          // two rows per lane iteration, both loads before either store
          for (int r = lane; r < L; r += 64) {
            const int r2 = r + 32;
            const bool two = r2 < L;
            const C x = col[r], x2 = two ? col[r2] : ew<C>::zero();
            const C v1 = v[r], v2 = two ? v[r2] : ew<C>::zero();
            col[r] = zfnma(v1, zc_, x);
            if (two) col[r2] = zfnma(v2, zc_, x2);
          }
        }
      }
      have_next = true;
      __syncthreads();
    }
    phase(3);
    // ---- 5. QR iteration on the packed matrix ---------------------------------
    C* Hq = Hg;
    if constexpr (QS) {
      // packed copy in shared memory (the vectors' region, no longer needed)
      Hq = zs;
      for (int c = 0; c < mp; ++c) {
        const int rmax = (c + 2 < mp - 1) ? c + 2 : mp - 1;
        const int64_t o = hess_coff(c, mp);
        for (int r = tid; r <= rmax; r += NTH) Hq[o + r] = (r <= c + 1) ? Hg[(size_t)c * ld + r] : ew<C>::zero();
      }
      __syncthreads();
    } else {
      // in-place repack of H (ld = mp) to the column-packed layout: a packed
      // offset never exceeds the unpacked one, so moving column by column in
      // increasing order through shared memory is safe
      for (int c = 0; c < mp; ++c) {
        const int rmax = (c + 2 < mp - 1) ? c + 2 : mp - 1;
        for (int r = tid; r <= rmax; r += NTH) v[r] = (r <= c + 1) ? Hg[(size_t)c * ld + r] : ew<C>::zero();
        __syncthreads();
        const int64_t o = hess_coff(c, mp);
        for (int r = tid; r <= rmax; r += NTH) Hg[o + r] = v[r];
        __syncthreads();
      }
    }
    phase(4);
    long long upd = 0;   // 2-element reflector applications (24 flops each), thread 0
    int st = qr_eigs<C, true>(SAcc<C>{Hq, mp}, mp, ev, s, s.refl, upd);
    flops += 24.0 * (double)upd;
    if (unscale != 1.0)
      for (int q = tid; q < mp; q += NTH) ev[q] = zscale(ev[q], unscale);
    phase(5);
    if (tid == 0) {
      status[inst] = st;
      if (flops_out) flops_out[inst] = flops;
    }
    __syncthreads();
  }
}
