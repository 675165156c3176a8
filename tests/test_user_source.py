"""USER source plug-ins (s-user.c) through the C ABI, on the CPU: a small
plug-in compiled here exercises argument splitting, the geometric area and
direction handed to user_open_source, energies kept or replaced, running
arrival times, the stop at a refused ray, user_start_iteration and
user_close_source."""
import os
import shutil
import subprocess

import numpy as np
import pytest

PLUGIN = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static int N, Limit, Iter;
static double Area, Px;
static FILE *Log;
int user_open_source (char **argv, int argc, double area, double px, double py, double pz)
{
   int i;
   Log = fopen (argv[0], "w");
   fprintf (Log, "argc=%d", argc);
   for (i = 0; i < argc; i++) fprintf (Log, " [%s]", argv[i]);
   fprintf (Log, " area=%g p=%g,%g,%g\n", area, px, py, pz);
   Limit = (argc > 1) ? atoi (argv[1]) : 5;
   Area = area; Px = px; N = 0;
   return 0;
}
int user_start_iteration (void) { return (Iter++ == 2) ? -1 : 0; }
int user_create_ray (double *t, double *energy, double *p1, double *p2, double *p3)
{
   if (N >= Limit) return -1;
   *p1 = -1.0; *p2 = 1e-4 * N; *p3 = -2e-4 * N;
   if (N % 2) *energy = 0.5 * N;           /* odd rays: the plug-in's energy */
   else if (N % 4 == 2) *energy = -1.0;    /* keep the spectrum's draw */
   if (N >= 2) *t = 0.25 * N;              /* no time for the first two rays */
   N++;
   return 0;
}
void user_close_source (void) { fprintf (Log, "closed\n"); fclose (Log); }
"""


@pytest.fixture(scope="module")
def plugin(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("user")
    (d / "src.c").write_text(PLUGIN)
    so = d / "libuser.so"
    subprocess.run([cc, "-shared", "-fPIC", "-o", str(so), str(d / "src.c")], check=True)
    return str(so), str(d / "log.txt")


def test_rays_energies_and_times(plugin):
    from marx_gb300.user_source import UserSource
    so, log = plugin
    s = UserSource(so, f"  {log}\t 7  extra ", geometric_area=1145.0, p=(-1.0, 0.001, -0.002))
    e = np.linspace(1.0, 2.0, 10)
    ph, times = s.create(e)
    assert ph.n == 7 and times                  # the plug-in refuses the eighth ray
    k = np.arange(7)
    np.testing.assert_array_equal(ph.p[0], -1.0)
    np.testing.assert_array_equal(ph.p[1], 1e-4 * k)
    np.testing.assert_array_equal(ph.energy, np.where(k % 2 == 1, 0.5 * k, e[:7]))
    # t = -1 for rays 0 and 1 (no time), then the running sum of 0.25 * k
    expect = np.zeros(7)
    run = 0.0
    for i in range(7):
        if i >= 2:
            run += 0.25 * i
            expect[i] = run
    np.testing.assert_array_equal(ph.arrival_time, expect)
    assert (ph.flags == 0).all()
    q, _ = s.create(e)                          # second iteration: the plug-in has run out of rays
    assert q.n == 0
    q, ts = s.create(e)                         # third: user_start_iteration says stop
    assert q.n == 0 and not ts
    s.close()
    text = open(log).read()
    assert text.startswith(f"argc=3 [{log}] [7] [extra] area=1145 p=-1,0.001,-0.002")
    assert text.rstrip().endswith("closed")


def test_missing_plugin_is_an_error(tmp_path):
    from marx_gb300.user_source import UserSource
    with pytest.raises(RuntimeError, match="Error linking"):
        UserSource(str(tmp_path / "none.so"))
