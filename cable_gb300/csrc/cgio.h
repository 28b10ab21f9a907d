// Binary container of the restart, forcing and output files: the binary
// equivalents of the reference's netCDF restart file (written by
// cable_output_impl.F90 write_restart :278-311, read by cable_initialise.F90
// get_restart_data :163-664), met file (cable_input.F90 get_met_data) and
// per-step output file.
//
// Layout (little-endian):
//   bytes 0..127     Header
//   bytes 128..      directory: nfields x 48-byte Entry (at most 82 fields)
//   bytes 4096..     nrecords records of record_bytes each; a record holds
//                    every field as one [width][mp] block in caller tile
//                    order, blocks 64-byte aligned, records 4096-byte aligned
// Host code only (no CUDA), so the format is usable and testable without a GPU.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cgio {

constexpr uint32_t kVersion = 1;
constexpr uint64_t kDataOffset = 4096;
constexpr uint32_t kMaxFields = (uint32_t)((kDataOffset - 128) / 48);

// element types (the public CABLEGPU_F32 / F64 / I32 / DF32 codes)
constexpr uint32_t kF32 = 0, kF64 = 1, kI32 = 2, kDF32 = 3;

struct Header {
  char magic[8];          // "CABLEGPU"
  uint32_t version;       // kVersion
  uint32_t kind;          // 1 restart, 2 forcing, 3 output
  uint64_t mp;            // tiles
  uint32_t nfields;
  uint32_t nrecords;
  int32_t ktau;           // restart: last completed step; forcing / output: first step
  int32_t doy0;           // day of year of the first forcing record
  float dels;             // step length (s)
  uint32_t reserved0;
  uint64_t data_offset;   // kDataOffset
  uint64_t record_bytes;  // bytes per record (a multiple of 4096)
  uint8_t reserved[64];
};
static_assert(sizeof(Header) == 128, "header is 128 bytes");

struct Entry {
  char name[32];          // NUL-padded
  uint32_t dtype;         // kF32 / kF64 / kI32 / kDF32 (two float words per value:
                          // `width` high rows, then `width` low rows)
  uint32_t width;         // rows (layers) of the field
  uint64_t offset;        // byte offset of the block within a record
};
static_assert(sizeof(Entry) == 48, "directory entry is 48 bytes");

// bytes of one [width][mp] block of `dtype` (before alignment)
uint64_t block_bytes(uint32_t dtype, uint32_t width, uint64_t mp);

struct File {
  int fd = -1;
  Header h{};
  std::vector<Entry> fields;
  std::string err;
};

// Creates `path` (truncating it) with the given fields (their offsets are
// computed here) and `nrecords` records of zeros.  0 or -1 with f.err set.
int create(File& f, const char* path, uint32_t kind, uint64_t mp, const std::vector<Entry>& fields,
           uint32_t nrecords, int32_t ktau, int32_t doy0, float dels);
// Opens and validates an existing file (magic, version, sizes, directory).
int open_read(File& f, const char* path);
int write_block(File& f, uint32_t rec, int field, const void* data);
int read_block(const File& f, uint32_t rec, int field, void* data);
// Reads the first `bytes` bytes of record `rec` (bytes <= record_bytes).
int read_record_prefix(const File& f, uint32_t rec, void* data, uint64_t bytes);
// index of the field called `name`, or -1
int find(const File& f, const char* name);
void close(File& f);

}  // namespace cgio
