/* TEST INFRASTRUCTURE ONLY.  Linked into the reference's benchmark harness
 * (tests/bench.c, tests/fftw-bench.c, libbench2/) when that harness is
 * compiled against this library's include/fftw3.h (make -C oracle harness):
 *   - plans are made in dry-run mode, so `--can-do <problem>` answers from
 *     this library's planner on a machine without a GPU;
 *   - the harness's planner hooks (tests/hook.c) inspect the reference's
 *     internal planner, which this library does not have: they are empty. */
#include "fftw3_gb300.h"

__attribute__((constructor)) static void gb_harness_dry_run(void) { fftw_gb300_set_dry_run(1); }

void install_hook(void);
void uninstall_hook(void);
void install_hook(void) {}
void uninstall_hook(void) {}
