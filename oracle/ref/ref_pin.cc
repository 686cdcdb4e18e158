// Exports the reference's own determinant, hash and alias-table routines with a C ABI so the
// oracle's restatement can be checked against them bit for bit.  Test infrastructure only.
#include <cstdint>
#include <vector>
#include "det.h"
#include "half_det.h"
#include "util.h"

static HalfDet make_half(uint64_t bits) {
  HalfDet h;
  for (unsigned o = 0; o < 64; o++)
    if (bits >> o & 1) h.set(o);
  return h;
}

extern "C" {

uint64_t ref_half_hash(uint64_t bits) { return make_half(bits).get_hash_value(); }

uint64_t ref_det_hash(uint64_t up, uint64_t dn) {
  Det d;
  d.up = make_half(up);
  d.dn = make_half(dn);
  return DetHasher()(d);
}

uint64_t ref_rehash(uint64_t a) { return Util::rehash(a); }

void ref_diff(uint64_t a, uint64_t b, unsigned* out, int* perm) {
  const DiffResult d = make_half(a).diff(make_half(b));
  out[0] = d.left_only[0];
  out[1] = d.left_only[1];
  out[2] = d.right_only[0];
  out[3] = d.right_only[1];
  out[4] = d.n_diffs;
  *perm = d.permutation_factor;
}

unsigned ref_n_diffs(uint64_t a, uint64_t b) { return make_half(a).n_diffs(make_half(b)); }

unsigned ref_bit_till(uint64_t a, unsigned p) { return make_half(a).bit_till(p); }

int ref_det_less(uint64_t ua, uint64_t da, uint64_t ub, uint64_t db) {
  Det a, b;
  a.up = make_half(ua);
  a.dn = make_half(da);
  b.up = make_half(ub);
  b.dn = make_half(db);
  return a < b ? 1 : 0;
}

void ref_alias(const double* probs, size_t n, double* new_probs, uint64_t* aliases) {
  std::vector<double> p(probs, probs + n), np;
  std::vector<size_t> al;
  Util::setup_alias_arrays(p, np, al);
  for (size_t i = 0; i < n; i++) {
    new_probs[i] = np[i];
    aliases[i] = al[i];
  }
}

}  // extern "C"
