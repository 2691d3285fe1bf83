// Compile check of the C++ adapters against ThunderEgg's own headers: every
// adapter class is instantiated for 2D and 3D.  Built with -fsyntax-only by
// tests/test_adapters.py (nothing is linked or run).
#include "thunderegg_gb300/adapters.hpp"

template class thunderegg_gb300::GpuDomain<2>;
template class thunderegg_gb300::GpuDomain<3>;
template class thunderegg_gb300::GpuGhostFiller<2>;
template class thunderegg_gb300::GpuGhostFiller<3>;
template class thunderegg_gb300::GpuStarPatchOperator<2>;
template class thunderegg_gb300::GpuStarPatchOperator<3>;
template class thunderegg_gb300::GpuDFTPatchSolver<2>;
template class thunderegg_gb300::GpuDFTPatchSolver<3>;
template class thunderegg_gb300::GpuLinearRestrictor<2>;
template class thunderegg_gb300::GpuLinearRestrictor<3>;
template class thunderegg_gb300::GpuDirectInterpolator<2>;
template class thunderegg_gb300::GpuDirectInterpolator<3>;
template class thunderegg_gb300::GpuVCycle<2>;
template class thunderegg_gb300::GpuVCycle<3>;
template class thunderegg_gb300::GpuBiCGStab<2>;
template class thunderegg_gb300::GpuBiCGStab<3>;
template class thunderegg_gb300::GpuCG<2>;
template class thunderegg_gb300::GpuCG<3>;
template class thunderegg_gb300::GpuBiCGStabPatchSolver<2>;
template class thunderegg_gb300::GpuBiCGStabPatchSolver<3>;
template class thunderegg_gb300::GpuCycle<2>;
template class thunderegg_gb300::GpuCycle<3>;
template class thunderegg_gb300::GpuCycleBuilder<2>;
template class thunderegg_gb300::GpuCycleBuilder<3>;
template class thunderegg_gb300::GpuIterativeRefinement<2>;
template class thunderegg_gb300::GpuIterativeRefinement<3>;
template thunderegg_gb300::LevelTables<2> thunderegg_gb300::flatten<2>(const ThunderEgg::Domain<2>&);
template thunderegg_gb300::LevelTables<3> thunderegg_gb300::flatten<3>(const ThunderEgg::Domain<3>&);
