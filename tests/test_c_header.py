"""The C ABI from plain C: include/cpab_gb300.h compiles as C99 (gcc -Wall
-Wextra -Werror), every function it declares links against the built
library, and the entry points that need no GPU behave as documented when
called from C (versions, cell counts, the ragged-image host plan, status
codes and messages for invalid arguments).  No CUDA call is made."""
import os
import re
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(REPO, 'libcpab_gb300')

PROGRAM = r'''
#include <stdio.h>
#include <string.h>
#include "cpab_gb300.h"

typedef void (*any_fn)(void);
static const any_fn every_entry_point[] = {
%(table)s
};

int main(void) {
    size_t i, n = sizeof every_entry_point / sizeof every_entry_point[0];
    for (i = 0; i < n; ++i)
        if (!every_entry_point[i]) return 2;
    printf("entry_points %%zu\n", n);
    printf("version %%d\n", cpab_version());
    {
        int nc2[2] = {3, 3}, nc3[3] = {4, 4, 4}, nc1[1] = {50};
        printf("cells %%d %%d %%d\n", cpab_num_cells(1, nc1), cpab_num_cells(2, nc2),
               cpab_num_cells(3, nc3));
    }
    {
        int sizes[2][2] = {{17, 23}, {224, 224}}, outsizes[2][2] = {{9, 40}, {224, 225}};
        long long plan[3 * CPAB_IMAGE_PLAN_FIELDS], tot[3];
        int rc = cpab_ragged_images_plan(2, 2, &sizes[0][0], &outsizes[0][0], plan, tot);
        printf("plan %%d %%lld %%lld %%lld %%lld %%lld\n", rc, tot[0], tot[1], tot[2],
               plan[CPAB_IMAGE_PLAN_FIELDS + 1], plan[CPAB_IMAGE_PLAN_FIELDS + 2]);
        sizes[1][0] = 0;
        rc = cpab_ragged_images_plan(2, 2, &sizes[0][0], NULL, plan, tot);
        printf("bad_size %%d %%s\n", rc, cpab_last_error());
    }
    {
        /* no work: returns before touching the device */
        int rc = cpab_interpolate_ragged(2, 0, 1, NULL, 0, 0, 0, NULL, NULL, NULL, NULL);
        printf("empty %%d\n", rc);
        rc = cpab_interpolate_ragged(4, 1, 1, NULL, 0, 0, 0, NULL, NULL, NULL, NULL);
        printf("bad_ndim %%d %%d\n", rc, (int)(strlen(cpab_last_error()) > 0));
        rc = cpab_interpolate_ragged(2, 1, 1, NULL, 16, 16, 1, NULL, NULL, NULL, NULL);
        printf("null_plan %%d\n", rc);
    }
    printf("codes %%d %%d %%d %%d %%d\n", CPAB_OK, CPAB_ERR_ARGUMENT, CPAB_ERR_CUDA,
           CPAB_ERR_UNSUPPORTED, CPAB_ERR_WORKSPACE);
    return 0;
}
'''


def _declared():
    src = open(os.path.join(REPO, 'include', 'cpab_gb300.h')).read()
    return sorted(set(re.findall(r'CPAB_API\s+[\w\s\*]*?\b(cpab_\w+)\s*\(', src)))


@pytest.fixture(scope='module')
def c_program(tmp_path_factory):
    gcc = shutil.which('gcc')
    lib = os.path.join(LIBDIR, 'libcpab_gb300.so')
    if not gcc or not os.path.exists(lib):
        pytest.skip('gcc or the built library is missing')
    d = tmp_path_factory.mktemp('cabi')
    names = _declared()
    table = ',\n'.join('    (any_fn)%s' % n for n in names)
    src = d / 'use_abi.c'
    src.write_text(PROGRAM % {'table': table})
    exe = d / 'use_abi'
    subprocess.check_call([gcc, '-std=c99', '-Wall', '-Wextra', '-Werror', '-O1',
                           '-I', os.path.join(REPO, 'include'), str(src), '-o', str(exe),
                           '-L', LIBDIR, '-lcpab_gb300', '-Wl,-rpath,' + LIBDIR])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    return dict(line.split(' ', 1) for line in out.stdout.strip().splitlines()), len(names)


def test_every_declared_function_links(c_program):
    res, n = c_program
    assert n >= 30
    assert res['entry_points'] == str(n)


def test_host_only_entry_points_from_c(c_program):
    res, _ = c_program
    assert int(res['version']) > 0
    assert res['cells'] == '50 36 320'
    # 17*23 + 224^2 data points, 9*40 + 224*225 output points, tiles 2*2 + 28*8
    # (8 x-rows x 32 last-axis columns per tile); image 1 starts at point 360, tile 4
    assert res['plan'] == '0 50567 50760 228 360 4'
    rc, msg = res['bad_size'].split(' ', 1)
    assert rc == '1' and 'image 1' in msg


def test_status_codes_from_c(c_program):
    res, _ = c_program
    assert res['empty'] == '0'
    assert res['bad_ndim'] == '1 1'
    assert res['null_plan'] == '1'
    assert res['codes'] == '0 1 2 3 4'
