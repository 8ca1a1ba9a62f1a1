// fault.h -- host-side fault injection for the library's device allocations (spk_debug_fail_allocation).
//
// Tests make an allocation fail on the host, the way a full device would answer, and check that every
// entry point reports SPK_ERR_OUT_OF_MEMORY and leaves its context usable; no GPU fault is involved.
#pragma once

namespace spk {

// Arms the injector: the nth device allocation from now fails once (0 disarms).
void fault_arm_allocation(unsigned nth);

// Called before every device allocation of the library; true when this one is to fail.
bool fault_allocation();

}  // namespace spk
