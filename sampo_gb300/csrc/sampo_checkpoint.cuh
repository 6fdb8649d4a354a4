// sampo_checkpoint.cuh - the checkpoint file of one simulation at a step
// boundary, shared by simulations (sampo_api.cu) and batch slots
// (sampo_batch.cu): a checkpoint of either loads into either.
//
//   header (CkHeader): magic "SAMPOCK1", version, the step about to run, the
//   carrying capacity, the population and its statistics, the counters the
//   next stats row reports, the slot count n; version 2 adds the population
//   at the previous step's start (the reference's stats line reads it,
//   src/abms.c:235-236), and a batch slot's device seed stream with the
//   coming step's seeds when they were already drawn;
//   then the nine 4-byte columns of slots [0, n) and their flag bytes.
#pragma once
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sampo_kernels.cuh"

namespace sampo {

constexpr char kCkMagic[8] = {'S', 'A', 'M', 'P', 'O', 'C', 'K', '1'};
enum : uint32_t { CK_PREV = 1u, CK_SEED_STREAM = 2u, CK_COMING_SEEDS = 4u };

struct CkHeader {
  char magic[8];
  uint32_t version, step;
  float cc;
  sampo_population pop;
  sampo_bites_cycles bnc;
  uint32_t n, flags;
  // version 2
  sampo_population prev;        // CK_PREV
  DevSeedStream rnd;            // CK_SEED_STREAM
  sampo_seeds coming[4];        // CK_COMING_SEEDS: the seeds of step `step`
};
constexpr size_t kCkHeaderV1 = offsetof(CkHeader, prev);

// Writes the header and slots [0, hd.n) of pool P; "" or an error message.
inline std::string ck_write(const char* path, const CkHeader& hd, const DevPool& P) {
  const size_t n = hd.n;
  std::vector<uint8_t> buf(n * 4 + 1);
  FILE* f = fopen(path, "wb");
  if (!f) return std::string("cannot write ") + path;
  bool ok = fwrite(&hd, sizeof(hd), 1, f) == 1;
  void* cols[9] = {P.age, P.his, P.delay, P.sporo, P.uni, P.avail, P.cycle, P.hbc, P.batches};
  for (int c = 0; c < 9 && ok; c++) {
    if (n && cudaMemcpy(buf.data(), cols[c], n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    if (ok && n) ok = fwrite(buf.data(), 4, n, f) == n;
  }
  if (ok && n && cudaMemcpy(buf.data(), P.flags, n, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
  if (ok && n) ok = fwrite(buf.data(), 1, n, f) == n;
  ok = (fclose(f) == 0) && ok;
  return ok ? std::string() : std::string("checkpoint write failed: ") + path;
}

// Reads the header (either version); the file stays open at the columns.
inline std::string ck_open(const char* path, CkHeader& hd, FILE** fp) {
  *fp = nullptr;
  FILE* f = fopen(path, "rb");
  if (!f) return std::string("cannot read ") + path;
  memset(&hd, 0, sizeof(hd));
  if (fread(&hd, kCkHeaderV1, 1, f) != 1 || memcmp(hd.magic, kCkMagic, 8) != 0 || (hd.version != 1 && hd.version != 2)) {
    fclose(f);
    return std::string("not a checkpoint: ") + path;
  }
  if (hd.version == 1) {
    hd.flags = 0;
  } else if (fread(reinterpret_cast<char*>(&hd) + kCkHeaderV1, sizeof(hd) - kCkHeaderV1, 1, f) != 1) {
    fclose(f);
    return std::string("short checkpoint header: ") + path;
  }
  if (hd.pop.r[7].end != hd.n) {
    fclose(f);
    return std::string("inconsistent checkpoint: ") + path;
  }
  *fp = f;
  return std::string();
}

// Reads the columns of hd.n slots into pool P and closes the file.
inline std::string ck_read_pool(FILE* f, const CkHeader& hd, const DevPool& P) {
  const size_t n = hd.n;
  std::vector<uint8_t> buf(n * 4 + 1);
  void* cols[9] = {P.age, P.his, P.delay, P.sporo, P.uni, P.avail, P.cycle, P.hbc, P.batches};
  bool ok = true;
  for (int c = 0; c < 9 && ok; c++) {
    ok = fread(buf.data(), 4, n, f) == n;
    if (ok && n) ok = cudaMemcpy(cols[c], buf.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (ok) ok = fread(buf.data(), 1, n, f) == n;
  if (ok && n) ok = cudaMemcpy(P.flags, buf.data(), n, cudaMemcpyHostToDevice) == cudaSuccess;
  fclose(f);
  return ok ? std::string() : std::string("checkpoint read failed");
}

}  // namespace sampo
