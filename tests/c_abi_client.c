/* A C client of include/vk_ros2.h: compiles a three-reaction network, reads
 * its table sizes and Jacobian pattern, and checks the error paths that need
 * no device (built and run by tests/test_capi_cpu.py). */
#include <stdio.h>
#include <string.h>

#include "vk_ros2.h"

#define CHECK(cond)                                            \
    do {                                                       \
        if (!(cond)) {                                         \
            printf("FAIL line %d: %s\n", __LINE__, #cond);     \
            return 1;                                          \
        }                                                      \
    } while (0)

int main(void) {
    /* species 0 H, 1 H2, 2 O, 3 OH; pairs:
     *   H + H + M <-> H2 + M,  O + H2 <-> OH + H,  OH + H <-> O + H2 */
    const int reac_ptr[] = {0, 3, 5, 7};
    const int reac_sp[] = {0, 0, -1, 2, 1, 3, 0};
    const int reac_nu[] = {1, 1, 1, 1, 1, 1, 1};
    const int prod_ptr[] = {0, 2, 4, 6};
    const int prod_sp[] = {1, -1, 3, 0, 2, 1};
    const int prod_nu[] = {1, 1, 1, 1, 1, 1};
    const double compo[] = {1, 0, /* H */ 2, 0, /* H2 */ 0, 1, /* O */ 1, 1 /* OH */};
    vk_network_desc d = {4, 3, reac_ptr, reac_sp, reac_nu, prod_ptr, prod_sp, prod_nu, 2, compo};
    vk_network *net = NULL;
    CHECK(vk_network_compile(&d, &net) == VK_OK && net != NULL);
    int nnz = 0, nw = 0, nsrc = 0;
    CHECK(vk_network_info(net, &nnz, &nw, &nsrc) == VK_OK);
    CHECK(nnz > 0 && nnz <= 16 && nw > 0 && nsrc > 0);
    int rows[16], cols[16];
    CHECK(vk_network_jac_pattern(net, rows, cols) == VK_OK);
    int diag = 0;
    for (int e = 0; e < nnz; ++e) {
        CHECK(rows[e] >= 0 && rows[e] < 4 && cols[e] >= 0 && cols[e] < 4);
        diag += rows[e] == cols[e];
    }
    CHECK(diag == 4); /* every species reacts, so every diagonal entry is stored */
    vk_network_free(net);

    /* a species index out of range is refused with a message */
    const int bad_sp[] = {0, 0, -1, 2, 1, 3, 99};
    d.reac_sp = bad_sp;
    net = NULL;
    CHECK(vk_network_compile(&d, &net) == VK_EINVAL && net == NULL);
    CHECK(strlen(vk_network_last_error()) > 0);

    /* calls on a NULL handle fail before any device work */
    CHECK(vk_run(NULL, NULL, 1, 1.0) == VK_EINVAL);
    CHECK(vk_get_state(NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL) == VK_EINVAL);
    CHECK(strlen(vk_last_error(NULL)) > 0);
    printf("c-abi ok: nnz %d, derivative terms %d, source terms %d\n", nnz, nw, nsrc);
    return 0;
}
