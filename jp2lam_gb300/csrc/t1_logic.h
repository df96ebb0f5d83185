// Bit-sliced Tier-1 context formation, shared by the modelling kernel and
// a host-side check.
//
// Every argument is a mask over samples (one bit per sample): bit i of `n`
// is set when sample i's north neighbour is significant, and so on. The
// functions form the zero-coding label (ISO/IEC 15444-1 Table D.1) and the
// sign-coding context and prediction bit (Table D.3) of all samples at once,
// as bit-planes, so a 64-bit mask forms 64 samples' contexts in a few dozen
// logic operations. jp2g_debug_context_labels evaluates them on single bits
// for every neighbourhood and the tests compare the result with the tables
// the rest of the coder uses.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define JP2G_HD __host__ __device__ __forceinline__
#else
#define JP2G_HD inline
#endif

namespace jp2g {

// Zero-coding label 0..8 as four bit-planes l[0..3] (l[0] least
// significant). orient: 0 LL, 1 HL, 2 LH, 3 HH (HL swaps the horizontal
// and vertical counts; HH keys on the diagonal count).
template <class M>
JP2G_HD void zc_label_planes(M nw, M n, M ne, M w, M e, M sw, M s, M se, int orient, M* l) {
  M h0 = w ^ e, h1 = w & e;  // horizontal count 0..2
  M v0 = n ^ s, v1 = n & s;  // vertical count 0..2
  const M a0 = nw ^ ne, a1 = nw & ne, b0 = sw ^ se, b1 = sw & se;
  const M d0 = a0 ^ b0, cy = a0 & b0;
  const M d1 = a1 ^ b1 ^ cy, d2 = (a1 & b1) | (cy & (a1 ^ b1));  // diagonal count 0..4
  M is8, is7, is6, is5, is4, is3, is2, is1;
  if (orient == 3) {
    const M hv0 = ~(h0 | h1 | v0 | v1);
    const M hv2 = h1 | v1 | (h0 & v0);  // h + v >= 2
    const M hv1 = ~hv0 & ~hv2;
    const M dz = ~(d0 | d1 | d2), dd1 = d0 & ~d1 & ~d2, dd2 = d1 & ~d0 & ~d2;
    is8 = d2 | (d1 & d0);
    is7 = dd2 & ~hv0;
    is6 = dd2 & hv0;
    is5 = dd1 & hv2;
    is4 = dd1 & hv1;
    is3 = dd1 & hv0;
    is2 = dz & hv2;
    is1 = dz & hv1;
  } else {
    if (orient == 1) {
      const M t0 = h0, t1 = h1;
      h0 = v0;
      h1 = v1;
      v0 = t0;
      v1 = t1;
    }
    const M hz = ~(h0 | h1), vz = ~(v0 | v1), dany = d0 | d1 | d2;
    is8 = h1;
    is7 = h0 & ~vz;
    is6 = h0 & vz & dany;
    is5 = h0 & vz & ~dany;
    is4 = hz & v1;
    is3 = hz & v0;
    is2 = hz & vz & (d1 | d2);
    is1 = hz & vz & d0 & ~d1 & ~d2;
  }
  l[3] = is8;
  l[2] = is7 | is6 | is5 | is4;
  l[1] = is7 | is6 | is3 | is2;
  l[0] = is7 | is5 | is3 | is1;
}

// Sign coding: n, s, w, e are the cardinal neighbours' significance, gn,
// gs, gw, ge their signs (1 = negative). The context is 9 + k (k 0..4); the
// returned planes m[0..2] are the three low bits of 9 + k - 8 = 1 + k, and x
// the sign-prediction bit that is XORed with the sample's own sign.
template <class M>
JP2G_HD void sign_planes(M n, M s, M w, M e, M gn, M gs, M gw, M ge, M* m, M* x) {
  const M hp = (w & ~gw) | (e & ~ge), hn = (w & gw) | (e & ge);
  const M vp = (n & ~gn) | (s & ~gs), vn = (n & gn) | (s & gs);
  const M hpos = hp & ~hn, hneg = hn & ~hp;  // horizontal contribution +1 / -1
  const M vpos = vp & ~vn, vneg = vn & ~vp;
  const M hz = ~(hpos | hneg), vz = ~(vpos | vneg);
  const M same = (hpos & vpos) | (hneg & vneg), opp = (hpos & vneg) | (hneg & vpos);
  const M k0 = hz & vz, k1 = hz & ~vz, k3 = ~hz & vz;
  m[0] = k0 | opp | same;  // k = 0, 2, 4
  m[1] = k1 | opp;         // k = 1, 2
  m[2] = k3 | same;        // k = 3, 4
  *x = hneg | (hz & vneg);
}

}  // namespace jp2g
