// Host check of the adaptive GMRES restart rule (gmres_restart.h): reads
// lines "m_min m_max step_min step_max m cr" from stdin and prints the next
// restart length for each; the test compares them with a restatement.
#include <cstdio>

#include "gmres_restart.h"

int main()
{
    mhfem::RestartRule R;
    int m = 0;
    double cr = 0;
    while (std::scanf("%d %d %d %d %d %lf", &R.m_min, &R.m_max, &R.step_min, &R.step_max, &m, &cr) == 6)
        std::printf("%d\n", mhfem::next_restart(m, cr, R));
    return 0;
}
