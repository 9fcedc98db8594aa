// Test infrastructure: prints, as hex, the bytes of the reference's
// Output_header_global (sfxc/include/output_header.h:70-97) filled the way
// Manager_node::send_global_header does (sfxc/src/manager_node.cc:670-703),
// from the fields given on the command line:
//   experiment year day seconds number_channels integration_us correlator_version
//   polarisation_type branch job_nr subjob_nr
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "output_header.h"

int main(int argc, char **argv) {
  if (argc != 12) {
    std::fprintf(stderr, "usage: %s experiment year day seconds nchan int_us version pol branch job subjob\n", argv[0]);
    return 2;
  }
  Output_header_global h;
  std::memset(&h, 0, sizeof(Output_header_global));
  h.header_size = sizeof(Output_header_global);
  std::strcpy(h.experiment, argv[1]);
  h.start_year = std::atoi(argv[2]);
  h.start_day = std::atoi(argv[3]);
  h.start_time = std::atoi(argv[4]);
  h.number_channels = std::atoi(argv[5]);
  h.integration_time = std::atoi(argv[6]);
  h.output_format_version = OUTPUT_FORMAT_VERSION;
  h.correlator_version = std::atoi(argv[7]);
  h.polarisation_type = std::atoi(argv[8]);
  std::strncpy(h.correlator_branch, argv[9], 15);
  h.correlator_branch[14] = 0;
  h.job_nr = std::atoi(argv[10]);
  h.subjob_nr = std::atoi(argv[11]);
  const unsigned char *b = reinterpret_cast<const unsigned char *>(&h);
  for (size_t i = 0; i < sizeof(h); i++) std::printf("%02x", b[i]);
  std::printf("\n");
  return 0;
}
