// Host-side check of the batched-launch bookkeeping (spd_batch.cuh): the
// block -> instance search over a block-offset table (including instances
// with no blocks), and the recorder that merges the i-th launch of every
// instance into one batched launch: per-site block offsets, argument packs
// in instance order, zero-fill ranges, and the errors for instances whose
// launch sequences differ.  Nothing is launched.  Exit status 0 when every
// check holds.
#include <cstdio>
#include <string>

#include "spd_batch.cuh"

using namespace spd_batch;

struct BodyA {
  static __device__ void run(spd::Blk, int, double*) {}
};
struct BodyB {
  static __device__ void run(spd::Blk, const double*) {}
};

static int failures = 0;
#define CHECK(cond)                                              \
  do {                                                           \
    if (!(cond)) {                                               \
      std::printf("FAILED line %d: %s\n", __LINE__, #cond);      \
      ++failures;                                                \
    }                                                            \
  } while (0)

int main() {
  // block -> instance, instance 1 and 3 without blocks
  const unsigned boff[] = {0, 3, 3, 10, 10, 11};
  const int n = 5;
  for (unsigned b = 0; b < 11; ++b) {
    const int i = instance_of(boff, n, b);
    CHECK(boff[i] <= b && b < boff[i + 1]);
  }
  CHECK(instance_of(boff, n, 0) == 0 && instance_of(boff, n, 2) == 0);
  CHECK(instance_of(boff, n, 3) == 2 && instance_of(boff, n, 9) == 2);
  CHECK(instance_of(boff, n, 10) == 4);

  // three instances, three launches each (A, zero-fill, B)
  double buf[3][4];
  const unsigned grids[3] = {5, 0, 7};
  BatchRec R;
  for (int i = 0; i < 3; ++i) {
    R.begin_instance(i == 0);
    R.add<BodyA>("a", dim3(grids[i]), dim3(128), 64, PackBuild<int, double*>::make(10 + i, buf[i]));
    R.add_zero(buf[i], 8 * (i + 1));
    R.add<BodyB>("b", dim3(1), dim3(32), 0, PackBuild<const double*>::make(static_cast<const double*>(buf[i])));
    CHECK(R.end_instance());
  }
  CHECK(R.err.empty());
  CHECK(R.sites.size() == 3);
  auto* a = dynamic_cast<Site<BodyA, int, double*>*>(R.sites[0].get());
  CHECK(a != nullptr);
  if (a) {
    CHECK(a->count() == 3);
    CHECK(a->boff[0] == 0 && a->boff[1] == 5 && a->boff[2] == 5 && a->boff[3] == 12);
    CHECK(a->packs[0].h == 10 && a->packs[1].h == 11 && a->packs[2].h == 12);
    CHECK(a->packs[2].r.h == buf[2]);
    CHECK(a->block.x == 128 && a->smem == 64);
  }
  auto* z = dynamic_cast<ZeroSite*>(R.sites[1].get());
  CHECK(z != nullptr);
  if (z) {
    CHECK(z->ranges.size() == 3 && z->ranges[1].bytes == 16 && z->ranges[2].p == (unsigned char*)buf[2]);
    CHECK(z->boff.back() == 3);  // one block per small range
  }
  auto* b = dynamic_cast<Site<BodyB, const double*>*>(R.sites[2].get());
  CHECK(b != nullptr && b->boff.back() == 3);

  // a second instance with another body where the first had BodyA
  {
    BatchRec S;
    S.begin_instance(true);
    S.add<BodyA>("a", dim3(2), dim3(128), 0, PackBuild<int, double*>::make(0, buf[0]));
    CHECK(S.end_instance());
    S.begin_instance(false);
    S.add<BodyB>("b", dim3(2), dim3(128), 0, PackBuild<const double*>::make(static_cast<const double*>(buf[0])));
    CHECK(!S.err.empty());
  }
  // same body, other block shape (another cells-per-block value)
  {
    BatchRec S;
    S.begin_instance(true);
    S.add<BodyA>("a", dim3(2), dim3(32, 4), 0, PackBuild<int, double*>::make(0, buf[0]));
    CHECK(S.end_instance());
    S.begin_instance(false);
    S.add<BodyA>("a", dim3(2), dim3(64, 4), 0, PackBuild<int, double*>::make(1, buf[1]));
    CHECK(!S.err.empty());
  }
  // fewer launches than the first instance
  {
    BatchRec S;
    S.begin_instance(true);
    S.add<BodyA>("a", dim3(2), dim3(32), 0, PackBuild<int, double*>::make(0, buf[0]));
    S.add_zero(buf[0], 8);
    CHECK(S.end_instance());
    S.begin_instance(false);
    S.add<BodyA>("a", dim3(2), dim3(32), 0, PackBuild<int, double*>::make(1, buf[1]));
    CHECK(!S.end_instance());
  }
  // a 2D grid cannot be merged
  {
    BatchRec S;
    S.begin_instance(true);
    S.add<BodyA>("a", dim3(2, 2), dim3(32), 0, PackBuild<int, double*>::make(0, buf[0]));
    CHECK(!S.err.empty());
  }
  std::printf("%s (%d failures)\n", failures ? "FAILED" : "ok", failures);
  return failures ? 1 : 0;
}
