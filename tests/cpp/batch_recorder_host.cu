// Host-side check of the batched-launch recorder (gevolution-1.2_gb300/csrc/gev_batch.cuh):
// no device call is made, so it runs without a GPU.  It records the launches of two
// bodies and a copy into a GevRecorder, as a context does while a cycle is recorded, and
// checks what the executor relies on:
//   - every argument pack starts on a 16-byte boundary of the recorder's byte buffer;
//   - a pack holds the body's parameters in order, converted to the body's parameter
//     types (the same conversions as an ordinary launch);
//   - a body's batched launcher is one function whatever the arguments, and two bodies
//     have two launchers (cohorts are formed on it);
//   - a launch with a 2-D grid marks the recording as not batchable;
//   - a copy keeps its host destination, device source and size.
// Prints "ok" and exits 0, or names the first failed check and exits 1.
#include <cstdio>
#include <cstring>

#include "../../gevolution-1.2_gb300/csrc/gev_batch.cuh"

__device__ void body_a(const float *p, long n, double x, int k) {}

struct Blob {
  int a;
  double b;
  float c[3];
};
__device__ void body_b(Blob s, const unsigned *q, unsigned char t) {}

static int fails = 0;
static void check(bool ok, const char *what) {
  if (!ok && fails++ == 0) printf("failed: %s\n", what);
}

int main() {
  float f = 0.f;
  unsigned u = 0u;
  GevRecorder r;
  r.add<body_a, 256, 1>(dim3(10), dim3(256), 0, &f, 5, 2.5f, 7L);  // int -> long, float -> double, long -> int
  const Blob blob{1, 2.0, {3.f, 4.f, 5.f}};
  r.add<body_b, 128, 2>(dim3(3), dim3(128), 64, blob, &u, 300);  // 300 -> unsigned char 44
  r.add_copy(&f, &u, 8);
  r.add<body_a, 256, 1>(dim3(10), dim3(256), 0, &f, 6L, 1.0, 8);

  check(r.ops.size() == 4, "four operations recorded");
  check(!r.bad, "one-dimensional grids keep the recording batchable");
  for (int k : {0, 1, 3}) check(r.ops[k].off % 16 == 0, "argument packs 16-byte aligned");

  typedef GevBodyArgs<decltype(&body_a)>::type PA;
  typedef GevBodyArgs<decltype(&body_b)>::type PB;
  check(r.ops[0].bytes == sizeof(PA) && r.ops[1].bytes == sizeof(PB), "pack sizes");
  PA pa;
  memcpy(&pa, r.args.data() + r.ops[0].off, sizeof(PA));
  check(pa.h == &f && pa.t.h == 5L && pa.t.t.h == 2.5 && pa.t.t.t.h == 7, "body_a's arguments, converted");
  PB pb;
  memcpy(&pb, r.args.data() + r.ops[1].off, sizeof(PB));
  check(pb.h.a == 1 && pb.h.b == 2.0 && pb.h.c[2] == 5.f && pb.t.h == &u && pb.t.t.h == 44,
        "body_b's arguments, converted");

  check(r.ops[0].launch != nullptr && r.ops[0].launch == r.ops[3].launch, "one launcher per body");
  check(r.ops[0].launch != r.ops[1].launch, "a launcher for each body");
  check(r.ops[1].grid.x == 3 && r.ops[1].block.x == 128 && r.ops[1].smem == 64, "grid, block and shared memory kept");

  check(r.ops[2].launch == nullptr && r.ops[2].dst == &f && r.ops[2].src == &u && r.ops[2].bytes == 8, "the copy");

  GevRecorder r2;
  r2.add<body_a, 256, 1>(dim3(4, 2), dim3(256), 0, &f, 1L, 1.0, 1);
  check(r2.bad, "a 2-D grid cannot be batched");

  r.clear();
  check(r.ops.empty() && r.args.empty() && !r.bad, "clear");
  if (fails) return 1;
  printf("ok\n");
  return 0;
}
