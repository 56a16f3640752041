// rtm_gb300_run: the reference's executable for the migrate path, on the
// GB300 engine.  Run in the directory the reference would run in; reads
// 2D_Real_RVSP_RTM.txt (or the run file given as the first argument) and the
// files it names, writes the per-shot and stacked images (rtm_run_config).
#include <cstdio>
#include <cstdlib>

#include "../../include/rtm_gb300.h"

int main(int argc, char **argv)
{
    const char *run_file = argc > 1 ? argv[1] : "2D_Real_RVSP_RTM.txt";
    const int max_batch = argc > 2 ? std::atoi(argv[2]) : 0;
    const int rc = rtm_run_config(run_file, max_batch);
    if (rc != RTM_OK) {
        std::fprintf(stderr, "rtm_gb300_run: %s (status %d)\n", rtm_last_error(), rc);
        return 1;
    }
    return 0;
}
