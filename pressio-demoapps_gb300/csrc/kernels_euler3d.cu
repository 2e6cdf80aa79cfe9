// Kernel instantiations and launchers for the Euler3d family.
#define PDA_FAM ::pda::Euler3d
#include "family_impl.cuh"

namespace pda {
const Launchers &launchers_euler3d() {
  static const Launchers L = {fam_impl::rows_velocity, fam_impl::struct_velocity,
                              fam_impl::struct_faces, fam_impl::struct_balance,
                              fam_impl::rows_vj_inner, fam_impl::rows_vj_nearbd,
                              fam_impl::batch_faces, fam_impl::batch_balance, fam_impl::batch_balance_stage,
                              fam_impl::batch_num_shapes, fam_impl::struct_vj,
                              fam_impl::lspg_fused,
                              fam_impl::lspg_fused_blocks, fam_impl::lspg_fused_prepare};
  return L;
}
}  // namespace pda
