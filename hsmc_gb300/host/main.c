/*
 * hsmc: the reference's command line (src/exec.c:28-145) over the GB300
 * engine.  -i/--input IN_FILE (default in.dat), -e/--example, -o/--output
 * OUT_FILE; dispatch on the input as the reference does: NpT when npt > 0,
 * else cavity sampling when cavity > 0, else cluster moves when cluster is
 * set, else NVT.
 */
#include <getopt.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hsmc_host.h"

static void usage(void) {
  printf("Usage: hsmc [-e] [-i IN_FILE] [-o OUT_FILE]\n"
         "hsmc performs Monte Carlo simulations of mono-disperse hard-sphere systems. \n"
         "The program is run as ./hsmc -i IN_FILE where IN_FILE is a file describing \n"
         "the parameters of the simulation. An example of input file can be obtained by \n"
         "running ./hsmc -e.\n\n"
         "  -e, --example              Print example of input file on screen\n"
         "  -i, --input=IN_FILE        Input read from IN_FILE instead of from  in.dat\n"
         "  -o, --output=OUT_FILE      Output to OUT_FILE instead of standard output\n");
}

int main(int argc, char **argv) {
  const char *input = "in.dat", *output = "";
  bool example = false;
  static const struct option opts[] = {{"input", required_argument, 0, 'i'},
                                       {"example", no_argument, 0, 'e'},
                                       {"output", required_argument, 0, 'o'},
                                       {"help", no_argument, 0, 'h'},
                                       {0, 0, 0, 0}};
  int c;
  while ((c = getopt_long(argc, argv, "i:eo:h", opts, NULL)) != -1) {
    switch (c) {
      case 'i': input = optarg; break;
      case 'e': example = true; break;
      case 'o': output = optarg; break;
      case 'h': usage(); return 0;
      default: usage(); return 64;
    }
  }
  if (argc - optind > 1) {
    usage();
    return 64;
  }
  if (example) host_print_example();
  if (strcmp(output, "") != 0 && !freopen(output, "w", stdout)) {
    printf("Failed to pipe output to file %s\n", output);
    exit(EXIT_FAILURE);
  }
  if (!example) {
    host_run run;
    memset(&run, 0, sizeof(run));
    host_read_input(&run.in, input);
    if (run.in.press > 0) {
      host_npt(&run);
    } else if (run.in.cavity_pcav > 0) {
      host_cavity(&run);
    } else if (run.in.cluster_flag > 0) {
      host_cluster(&run);
    } else {
      host_nvt(&run);
    }
    printf("Simulation complete!\n");
  }
  return 0;
}
