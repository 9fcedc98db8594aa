// Process-level symbols the reference's correlator-node classes expect from
// sfxc/src/utils.cc and MPI, supplied for a single-process CPU checker
// (test infrastructure only).  Assertions abort the checker process, which is
// how the reference treats them (sfxc/src/utils.cc:44-90).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mpi.h"

int RANK_OF_NODE = 0;
std::string ID_OF_NODE;
std::string HOSTNAME_OF_NODE;

void abort_sfxc_assertion(const char *file, int line, const char *message) {
  std::fprintf(stderr, "reference assertion failed: %s:%d: %s\n", file, line, message);
  std::abort();
}

void sfxc_abort(const char *msg) {
  std::fprintf(stderr, "reference abort: %s\n", msg ? msg : "");
  std::abort();
}

// Messages "sent" by the checked code, in order (tag, bytes).
struct ShimMessage {
  int tag;
  std::vector<char> bytes;
};
std::vector<ShimMessage> g_shim_messages;

static int type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_SHORT: return 2;
    case MPI_INT: return 4;
    case MPI_FLOAT: return 4;
    case MPI_LONG_LONG: return 8;
    case MPI_DOUBLE: return 8;
    default: return 1;
  }
}

extern "C" int MPI_Pack(const void *inbuf, int incount, MPI_Datatype datatype, void *outbuf,
                        int outsize, int *position, MPI_Comm) {
  int n = incount * type_size(datatype);
  if (*position + n > outsize) sfxc_abort("MPI_Pack overflow");
  std::memcpy((char *)outbuf + *position, inbuf, n);
  *position += n;
  return MPI_SUCCESS;
}

extern "C" int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int, int tag, MPI_Comm) {
  ShimMessage m;
  m.tag = tag;
  m.bytes.assign((const char *)buf, (const char *)buf + count * type_size(datatype));
  g_shim_messages.push_back(m);
  return MPI_SUCCESS;
}

extern "C" int MPI_Comm_size(MPI_Comm, int *size) {
  *size = 1;
  return MPI_SUCCESS;
}

extern "C" int MPI_Comm_rank(MPI_Comm, int *rank) {
  *rank = 0;
  return MPI_SUCCESS;
}

// Modified Julian Day of a Gregorian calendar date, the helper that
// sfxc/src/utils.cc:255 provides to the format readers (VDIF epochs).  Own
// formulation: days since 0000-03-01 of the proleptic Gregorian calendar,
// minus that count for 1858-11-17.
int mjd(int day, int month, int year) {
  const int y = year - (month <= 2 ? 1 : 0);
  const int era = (y >= 0 ? y : y - 399) / 400;
  const int yoe = y - era * 400;
  const int mp = (month + 9) % 12;
  const int doy = (153 * mp + 2) / 5 + day - 1;
  const int doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + doe - 678881;
}
