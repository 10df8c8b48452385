// Enhanced-assumed-strain Q1 hexahedra with the hyperelastic framework's laws (Hyperelastic<Deviatoric<DF>,
// Volumetric<VF>>, materials/hyperelastic/interface.hh): the element kernel of element_eas.cuh instantiated with the
// material point of hyperelastic.cuh, in its own translation unit so the closed-form laws' kernels keep their
// register allocation.
#include "element_eas.cuh"

namespace ikr {

void launch_eas_element_hyper(const ElemArgs& a, int mode, bool fp32, const int32_t* list, int n, int base,
                              cudaStream_t s) {
  launch_eas_family<true>(a, mode, fp32, list, n, base, s);
}

}  // namespace ikr
