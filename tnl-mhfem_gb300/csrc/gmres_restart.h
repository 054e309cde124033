// Adaptive restart length of GMRES(m), host side.
//
// The reference's example configuration varies the restart length between
// gmres-restarting-min and gmres-restarting-max in steps between
// gmres-restarting-step-min and gmres-restarting-step-max
// (examples/HeatEquation/config.ini: 3, 30, 2, 4).  The rule that applies
// them lives in TNL's GMRES, which is not in the reference tree; this
// restates the published strategy those keys parametrize (A. H. Baker,
// E. R. Jessup, Tz. V. Kolev, "A simple strategy for varying the restart
// parameter in GMRES(m)", J. Comput. Appl. Math. 230 (2009) 751-761).  With
// cr = ||r_j|| / ||r_{j-1}||, the ratio of the true residual norms at two
// consecutive restarts (applied between cycles by the host, or inside the
// persistent small-system solve by the device: next_restart_with):
//  - cr > cos(8 deg) (the last cycle stagnated): m = m_max;
//  - cr < cos(80 deg) (it converged well): m stays;
//  - otherwise m decreases by the step d, and wraps to m_max when it would
//    fall below m_min.
// The paper keeps d fixed.  Here d is step_max when the cycle reduced the
// residual by more than the middle of that band (cr below the mean of the
// two cosines) and step_min otherwise, so the length shrinks faster while
// the cycles still converge well; with step_min == step_max this is the
// paper's rule.  The first cycle runs m_max.
//
// The header compiles as plain C++ too, so the host test suite checks the
// rule against a restatement.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define MHFEM_RESTART_HD __host__ __device__ __forceinline__
#else
#define MHFEM_RESTART_HD inline
#endif

namespace mhfem {

struct RestartRule {
    int m_min = 0, m_max = 30;       // m_min == 0 or m_min >= m_max: fixed at m_max
    int step_min = 0, step_max = 0;  // step_min <= 0: fixed at m_max
};

MHFEM_RESTART_HD bool restart_adaptive(const RestartRule& R)
{
    return R.m_min > 0 && R.m_min < R.m_max && R.step_min > 0;
}

// The two thresholds of the rule, cos 8 deg and cos 80 deg.
inline double restart_max_cr() { return std::cos(8.0 * 3.14159265358979323846 / 180.0); }
inline double restart_min_cr() { return std::cos(80.0 * 3.14159265358979323846 / 180.0); }

// Restart length of the next cycle after a cycle of length m whose restart
// residual ratio was cr, with the thresholds given (the device takes them
// from its state, computed here on the host).
MHFEM_RESTART_HD int next_restart_with(int m, double cr, const RestartRule& R, double max_cr, double min_cr)
{
    if (!restart_adaptive(R)) return R.m_max;
    if (!(cr <= max_cr)) return R.m_max;  // stagnation (or a non-finite ratio)
    if (cr < min_cr) return m;
    const int step_max = R.step_max > R.step_min ? R.step_max : R.step_min;
    const int d = cr < 0.5 * (min_cr + max_cr) ? step_max : R.step_min;
    return m - d >= R.m_min ? m - d : R.m_max;
}

inline int next_restart(int m, double cr, const RestartRule& R)
{
    return next_restart_with(m, cr, R, restart_max_cr(), restart_min_cr());
}

}  // namespace mhfem
