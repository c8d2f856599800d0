/* A C99 caller of the library's host-only entry points: the header compiles
 * as C and the symbols link without C++ or Python. */
#include <stdio.h>
#include <string.h>

#include "mcd.h"

int main(void) {
    mcd_material m;
    if (mcd_abi_version() != MCD_ABI_VERSION) return 1;
    if (mcd_material_init("Au", &m) != MCD_OK || m.Z != 79 || m.n_shells != 8) return 2;
    if (mcd_material_init("Fe", &m) != MCD_ENOSPECIES) return 3;
    if (mcd_struct_size("mcd_sim") != sizeof(mcd_sim)) return 4;
    if (mcd_struct_size("mcd_tally") != sizeof(mcd_tally)) return 5;
    if (mcd_event_bytes(0) != sizeof(mcd_event)) return 6;
    if (mcd_event_bytes(MCD_EV_PATHL | MCD_EV_W | MCD_EV_C2 | MCD_EV_POS | MCD_EV_PACKED_HEAD) != 28) return 7;
    if (mcd_sigma_table_bytes() != (size_t)1 << 20) return 8;
    if (strcmp(mcd_strerror(MCD_EINVAL), "invalid argument") != 0) return 9;
    printf("ok %d\n", mcd_abi_version());
    return 0;
}
