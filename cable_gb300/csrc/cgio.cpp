// Binary restart / forcing / output container (layout in cgio.h).
#include "cgio.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstring>

#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "the container is little-endian; a big-endian host would need byte swapping"
#endif

namespace cgio {
namespace {

constexpr char kMagic[8] = {'C', 'A', 'B', 'L', 'E', 'G', 'P', 'U'};

uint64_t round_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

int fail(File& f, const std::string& what) {
  f.err = what;
  if (errno) f.err += std::string(": ") + std::strerror(errno);
  return -1;
}

// full-length pread / pwrite (they may return short counts)
bool pread_all(int fd, void* buf, uint64_t n, uint64_t off) {
  char* p = (char*)buf;
  while (n > 0) {
    ssize_t r = ::pread(fd, p, n, (off_t)off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r; n -= (uint64_t)r; off += (uint64_t)r;
  }
  return true;
}
bool pwrite_all(int fd, const void* buf, uint64_t n, uint64_t off) {
  const char* p = (const char*)buf;
  while (n > 0) {
    ssize_t r = ::pwrite(fd, p, n, (off_t)off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r; n -= (uint64_t)r; off += (uint64_t)r;
  }
  return true;
}

}  // namespace

uint64_t block_bytes(uint32_t dtype, uint32_t width, uint64_t mp) {
  const uint64_t es = (dtype == kF64 || dtype == kDF32) ? 8 : 4;
  return es * width * mp;
}

int create(File& f, const char* path, uint32_t kind, uint64_t mp, const std::vector<Entry>& fields,
           uint32_t nrecords, int32_t ktau, int32_t doy0, float dels) {
  errno = 0;
  f = File();
  if (!path || mp == 0 || fields.empty() || fields.size() > kMaxFields) return fail(f, "create: bad argument");
  f.fields = fields;
  uint64_t off = 0;
  for (Entry& e : f.fields) {
    if (e.dtype > kDF32 || e.width == 0 || e.name[sizeof(e.name) - 1] != '\0') return fail(f, "create: bad field");
    e.offset = off;
    off = round_up(off + block_bytes(e.dtype, e.width, mp), 64);
  }
  std::memset(&f.h, 0, sizeof(f.h));
  std::memcpy(f.h.magic, kMagic, 8);
  f.h.version = kVersion;
  f.h.kind = kind;
  f.h.mp = mp;
  f.h.nfields = (uint32_t)f.fields.size();
  f.h.nrecords = nrecords;
  f.h.ktau = ktau;
  f.h.doy0 = doy0;
  f.h.dels = dels;
  f.h.data_offset = kDataOffset;
  f.h.record_bytes = round_up(off, 4096);
  f.fd = ::open(path, O_CREAT | O_TRUNC | O_RDWR, 0644);
  if (f.fd < 0) return fail(f, std::string("create: cannot open ") + path);
  std::vector<char> head(kDataOffset, 0);
  std::memcpy(head.data(), &f.h, sizeof(f.h));
  std::memcpy(head.data() + sizeof(f.h), f.fields.data(), f.fields.size() * sizeof(Entry));
  if (!pwrite_all(f.fd, head.data(), head.size(), 0)) return fail(f, "create: header write failed");
  // size the file so unwritten records read as zeros
  if (::ftruncate(f.fd, (off_t)(kDataOffset + f.h.record_bytes * (uint64_t)nrecords)) != 0)
    return fail(f, "create: cannot size the file");
  return 0;
}

int open_read(File& f, const char* path) {
  errno = 0;
  f = File();
  if (!path) return fail(f, "open: null path");
  f.fd = ::open(path, O_RDONLY);
  if (f.fd < 0) return fail(f, std::string("open: cannot open ") + path);
  if (!pread_all(f.fd, &f.h, sizeof(f.h), 0)) return fail(f, "open: short header");
  errno = 0;
  if (std::memcmp(f.h.magic, kMagic, 8) != 0) return fail(f, "open: not a CABLEGPU file (bad magic)");
  if (f.h.version != kVersion) return fail(f, "open: unsupported version");
  if (f.h.nfields == 0 || f.h.nfields > kMaxFields || f.h.mp == 0 || f.h.data_offset != kDataOffset)
    return fail(f, "open: corrupt header");
  f.fields.resize(f.h.nfields);
  if (!pread_all(f.fd, f.fields.data(), f.fields.size() * sizeof(Entry), sizeof(Header)))
    return fail(f, "open: short directory");
  errno = 0;
  for (const Entry& e : f.fields) {
    if (e.dtype > kDF32 || e.width == 0 || e.name[sizeof(e.name) - 1] != '\0' ||
        e.offset + block_bytes(e.dtype, e.width, f.h.mp) > f.h.record_bytes)
      return fail(f, "open: corrupt directory");
  }
  struct stat st;
  if (::fstat(f.fd, &st) != 0) return fail(f, "open: stat failed");
  errno = 0;
  if ((uint64_t)st.st_size < kDataOffset + f.h.record_bytes * (uint64_t)f.h.nrecords)
    return fail(f, "open: file shorter than its records (truncated)");
  return 0;
}

int write_block(File& f, uint32_t rec, int field, const void* data) {
  errno = 0;
  if (f.fd < 0 || field < 0 || field >= (int)f.fields.size() || rec >= f.h.nrecords || !data)
    return fail(f, "write: bad argument");
  const Entry& e = f.fields[field];
  const uint64_t off = kDataOffset + f.h.record_bytes * rec + e.offset;
  if (!pwrite_all(f.fd, data, block_bytes(e.dtype, e.width, f.h.mp), off)) return fail(f, "write failed");
  return 0;
}

int read_block(const File& f, uint32_t rec, int field, void* data) {
  if (f.fd < 0 || field < 0 || field >= (int)f.fields.size() || rec >= f.h.nrecords || !data) return -1;
  const Entry& e = f.fields[field];
  const uint64_t off = kDataOffset + f.h.record_bytes * rec + e.offset;
  return pread_all(f.fd, data, block_bytes(e.dtype, e.width, f.h.mp), off) ? 0 : -1;
}

int read_record_prefix(const File& f, uint32_t rec, void* data, uint64_t bytes) {
  if (f.fd < 0 || rec >= f.h.nrecords || !data || bytes > f.h.record_bytes) return -1;
  return pread_all(f.fd, data, bytes, kDataOffset + f.h.record_bytes * rec) ? 0 : -1;
}

int find(const File& f, const char* name) {
  for (size_t i = 0; i < f.fields.size(); ++i)
    if (std::strncmp(f.fields[i].name, name, sizeof(f.fields[i].name)) == 0) return (int)i;
  return -1;
}

void close(File& f) {
  if (f.fd >= 0) ::close(f.fd);
  f.fd = -1;
}

}  // namespace cgio
