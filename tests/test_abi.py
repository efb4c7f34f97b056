"""The C-ABI boundary without a GPU: the library builds, loads and exports
every entry point include/ug4gb.h declares; calls fail with status codes
(no exception, no crash) when no device is present; the header compiles as
C; the C++ adapter layer compiles against the header."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ug4gb.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"UG4GB_API\s+[\w\s\*]*?\b(ug4gb_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    assert len(names) >= 60
    from ugcore_gb300 import _lib
    assert set(names) == set(_lib.exported_symbols()), set(names) ^ set(_lib.exported_symbols())


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(ug4gb_\w+)", out))
    missing = set(declared()) - exported
    assert not missing, missing
    lib = ctypes.CDLL(built_lib)
    for n in declared():
        assert getattr(lib, n)


def test_calls_without_device_return_status(built_lib):
    from ugcore_gb300 import _lib
    L = _lib.lib()
    h = ctypes.c_void_p()
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc = L.ug4gb_create(0, ctypes.byref(h))
    assert rc < 0 and not h.value
    # null handles are rejected, not dereferenced
    assert L.ug4gb_vector_set(None, 1.0) == _lib.ERR_INVALID
    assert L.ug4gb_solver_init(None, None) == _lib.ERR_INVALID
    assert L.ug4gb_gmg_apply(None, None, None) == _lib.ERR_INVALID
    assert L.ug4gb_last_error(None) == b"null context"


def test_header_is_plain_c(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    src = tmp_path / "t.c"
    src.write_text('#include "ug4gb.h"\nint main(void){ ug4gb_ctx *c = 0; return ug4gb_create(0, &c) == 12345; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_adapter_compiles_and_links(built_lib, tmp_path):
    cxx = shutil.which("g++")
    src = tmp_path / "a.cpp"
    src.write_text(r'''
#include "ug4gb.hpp"
#include <cstdio>
int main() {
    try {
        ug4gb::Context ctx(0);
        ug4gb::Grid g(ctx, UG4GB_HEX, 2, 2, 2, 2);
        ug4gb::Disc d(ctx, g);
        d.set_diffusion(1.0);
        d.set_source_uniform(1);
        int top = g.num_levels() - 1;
        ug4gb::Matrix A(ctx.get());
        ug4gb::Vector b(ctx.get(), g.num_vertices(top)), x(ctx.get(), g.num_vertices(top));
        d.assemble_linear(top, A, b);
        ug4gb::GMG gmg(ctx, d);
        gmg.set_smoother(UG4GB_SMOOTHER_JACOBI, 0.6);
        gmg.init(A);
        ug4gb::Solver cg(ctx, UG4GB_SOLVER_CG);
        cg.set_preconditioner(&gmg);
        cg.set_convergence_check(100, 1e-300, 1e-10);
        cg.init(A);
        bool ok = cg.apply(x, b);
        std::printf("steps %d ok %d\n", cg.steps(), (int)ok);
        return ok ? 0 : 3;
    } catch (const ug4gb::Error &e) {
        std::printf("error %d: %s\n", e.code(), e.what());
        return 2;
    }
}
''')
    exe = tmp_path / "a.out"
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "ugcore_gb300", "adapters"), str(src), built_lib,
                        "-Wl,-rpath," + os.path.dirname(built_lib), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    import torch
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    if torch.cuda.is_available():
        assert r.returncode == 0 and "ok 1" in r.stdout, r.stdout + r.stderr
    else:
        assert r.returncode == 2 and "error" in r.stdout


def test_ugcore_glue_instantiates_reference_solvers(tmp_path):
    """The ugcore-side GPU algebra (ugcore_gb300/adapters/ug4gb_algebra.h)
    compiles against ugcore's own headers, ugcore's CG, BiCGStab,
    LinearSolver and MatrixOperator templates instantiate with its types, and
    ugcore's CG takes the library's multigrid (ug4gb_preconditioner.h) as its
    ILinearIterator preconditioner (where the ugcore tree is present; four
    empty stand-ins replace headers that need Boost)."""
    from helpers import reference_tree
    ref = reference_tree()
    if ref is None:
        pytest.skip("ugcore source tree not present")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    shim = tmp_path / "shim"
    for h in ("lib_disc/function_spaces/approximation_space.h", "lib_disc/common/function_group.h",
              "boost/graph/adjacency_list.hpp", "boost/graph/graph_traits.hpp"):
        (shim / h).parent.mkdir(parents=True, exist_ok=True)
        (shim / h).write_text("")
    src = tmp_path / "glue.cpp"
    src.write_text(r'''
#include "ug4gb_algebra.h"
#include "ug4gb_preconditioner.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/linear_solver/cg.h"
#include "lib_algebra/operator/linear_solver/bicgstab.h"
#include "lib_algebra/operator/linear_solver/linear_solver.h"
template class ug::CG<ug::GPUAlgebra::vector_type>;
template class ug::BiCGStab<ug::GPUAlgebra::vector_type>;
template class ug::LinearSolver<ug::GPUAlgebra::vector_type>;
template class ug::MatrixOperator<ug::GPUAlgebra::matrix_type, ug::GPUAlgebra::vector_type>;
static_assert(ug::GPUAlgebra::blockSize == 1, "scalar algebra");
// the rest of the matrix / vector interface the algebra templates call
void use(ug::UG4GBSparseMatrix &A, const ug::UG4GBSparseMatrix &B, ug::UG4GBVector &v, const ug::UG4GBVector &w)
{
    A.resize_and_clear(4, 4);
    A.set_as_copy_of(B, 2.0);
    A.scale(0.5);
    A.clear_retain_structure();
    A.apply_ignore_zero_rows(v, 1.0, w);
    double a = A(0, 1) + v.maxnorm() + w[2];
    v.set_value(0, a);
    A.add_entries({0}, {0}, {1.0});
}
// ugcore's CG with the library's multigrid as its preconditioner
bool solve(ug4gb_disc *disc, SmartPtr<ug::MatrixOperator<ug::UG4GBSparseMatrix, ug::UG4GBVector> > A,
           ug::UG4GBVector &u, ug::UG4GBVector &b)
{
    SmartPtr<ug::UG4GBGeometricMultiGrid> gmg = make_sp(new ug::UG4GBGeometricMultiGrid(disc));
    gmg->set_smoother(UG4GB_SMOOTHER_JACOBI, 0.6);
    gmg->set_precision("mixed");
    ug::CG<ug::UG4GBVector> cg;
    cg.set_preconditioner(gmg);
    cg.init(A);
    return cg.apply(u, b);
}
int main() { return ug::GPUAlgebra::get_type().type() == ug::AlgebraType::GPU ? 0 : 1; }
''')
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-w", "-I" + str(shim), "-I" + os.path.join(ref, "ugbase"),
                        "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "ugcore_gb300", "adapters"),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_ugcore_cg_drives_the_library_at_run_time(tmp_path):
    """An executable from ugcore's own CG, StdConvCheck and MatrixOperator
    (headers of the reference tree) over the GPU algebra and multigrid,
    linked with ugcore's common/ objects (built by oracle/build_ref.sh from
    the reference sources) and libug4gb.so: it assembles the 17^3 hex
    Poisson problem through the C ABI and solves it with ugcore's CG and the
    library's multigrid.  Where a GPU is present it must converge; without
    one it must stop at the first device call with ugcore's error type
    (UGError, exit 2) and the library's message."""
    from helpers import reference_tree
    from ugcore_gb300 import build
    ref = reference_tree()
    if ref is None:
        pytest.skip("ugcore source tree not present")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    r = subprocess.run(["sh", os.path.join(ROOT, "oracle", "build_ref.sh")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    obj = os.path.join(ROOT, "oracle", "_ref", "obj")
    objs = [os.path.join(obj, o) for o in ("common_log.o", "common_debug_id.o", "common_assert.o", "common_error.o",
                                           "common_progress.o", "common_util_string_util.o",
                                           "common_util_ostream_buffer_splitter.o", "crc32_stub.o")]
    for o in objs:
        assert os.path.exists(o), o
    lib = build.build()
    src = tmp_path / "run.cpp"
    src.write_text(r'''
#include <cstdio>
#include "ug4gb_algebra.h"
#include "ug4gb_preconditioner.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/linear_solver/cg.h"
#include "lib_algebra/operator/convergence_check.h"
using namespace ug;
typedef MatrixOperator<UG4GBSparseMatrix, UG4GBVector> Op;
int main()
{
    try {
        SmartPtr<Op> A = make_sp(new Op);                       // first device call: the engine context
        ug4gb_ctx *ctx = ug4gb_glue::context().get();
        ug4gb_grid *g = nullptr;
        ug4gb_disc *d = nullptr;
        ug4gb::check(ug4gb_grid_create_structured(ctx, UG4GB_HEX, 2, 2, 2, 3, &g), ctx, "grid");
        ug4gb::check(ug4gb_disc_create(ctx, g, &d), ctx, "disc");
        ug4gb::check(ug4gb_disc_set_diffusion_constant(d, 1.0), ctx, "diffusion");
        ug4gb::check(ug4gb_disc_set_source_uniform(d, 1), ctx, "source");
        const int top = ug4gb_grid_num_levels(g) - 1;
        int n = 0;
        ug4gb::check(ug4gb_grid_level_info(g, top, &n, nullptr, nullptr, nullptr), ctx, "level");
        UG4GBVector u(n), b(n);
        ug4gb::check(ug4gb_disc_assemble_linear(d, top, A->impl().get(), b.impl().get()), ctx, "assemble");
        SmartPtr<UG4GBGeometricMultiGrid> gmg = make_sp(new UG4GBGeometricMultiGrid(d));
        gmg->set_smoother(UG4GB_SMOOTHER_JACOBI, 0.6);
        CG<UG4GBVector> cg;                                      // ugcore's own CG (cg.h)
        cg.set_preconditioner(gmg);
        cg.set_convergence_check(make_sp(new StdConvCheck<UG4GBVector>(100, 1e-50, 1e-10, false)));
        cg.init(A);
        u.set(0.0);
        const bool ok = cg.apply(u, b);
        std::printf("ok %d steps %d\n", ok ? 1 : 0, cg.step());
        return ok ? 0 : 1;
    } catch (const UGError &e) {
        std::printf("error: %s\n", e.get_msg().c_str());
        return 2;
    }
}
''')
    shim = os.path.join(ROOT, "oracle", "_ref", "shim")
    exe = tmp_path / "run"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-w", "-I" + shim, "-I" + os.path.join(ref, "ugbase"),
                        "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "ugcore_gb300", "adapters"),
                        str(src)] + objs + [lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    import torch
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    if torch.cuda.is_available():
        assert r.returncode == 0 and "ok 1" in r.stdout, r.stdout + r.stderr
    else:
        assert r.returncode == 2 and r.stdout.startswith("error:") and "UG4GBSparseMatrix" in r.stdout, \
            r.stdout + r.stderr


BOOST_STANDIN_HEADERS = [
    "boost/mpl/at.hpp", "boost/mpl/empty.hpp", "boost/mpl/fold.hpp", "boost/mpl/for_each.hpp", "boost/mpl/front.hpp",
    "boost/mpl/if.hpp", "boost/mpl/list.hpp", "boost/mpl/map.hpp", "boost/mpl/min_max.hpp", "boost/mpl/pop_front.hpp",
    "boost/mpl/size.hpp", "boost/mpl/transform_view.hpp", "boost/optional.hpp", "boost/serialization/access.hpp",
    "boost/serialization/export.hpp", "boost/serialization/level.hpp", "boost/serialization/nvp.hpp",
    "boost/serialization/version.hpp"]


@pytest.mark.parametrize("negative", [False, True])
def test_ugcore_bridge_compiles_against_ugcore_headers(tmp_path, negative):
    """The ugcore-side bridge -- UG4GBDomainDiscretization as ugcore's
    IDomainDiscretization<GPUAlgebra> (ug4gb_domain_disc.h), the multigrid on
    it (ug4gb_preconditioner.h) and the registration RegisterUG4GB /
    InitUGPlugin_UG4GB (ug4gb_bridge.cpp) -- compiles against ugcore's own
    lib_disc, lib_grid, registry and bridge headers for 2D and 3D domains
    (both instantiated), with the Boost headers they name replaced by the
    stand-in tests/standins/boost/ug_boost_standin.hpp (Boost is absent).
    The negative case plants a wrong call in a copy of the adapter to show
    that the instantiated code is checked."""
    from helpers import reference_tree
    ref = reference_tree()
    if ref is None:
        pytest.skip("ugcore source tree not present")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    shim = tmp_path / "shim"
    for h in BOOST_STANDIN_HEADERS:
        (shim / h).parent.mkdir(parents=True, exist_ok=True)
        (shim / h).write_text('#include "boost/ug_boost_standin.hpp"\n')
    src_dir = os.path.join(ROOT, "ugcore_gb300", "adapters")
    if negative:
        work = tmp_path / "adapters"
        shutil.copytree(src_dir, work)
        dd = work / "ug4gb_domain_disc.h"
        txt = dd.read_text()
        bad = txt.replace("ug4gb_disc_adjust_solution(m_disc, m_top, m_u->get())",
                          "ug4gb_disc_adjust_solution(m_disc, m_top, m_u->get(), 1)")
        assert bad != txt
        dd.write_text(bad)
        src_dir = str(work)
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-w", "-DUG_DIM_2", "-DUG_DIM_3", "-I" + str(shim),
                        "-I" + os.path.join(ROOT, "tests", "standins"), "-I" + os.path.join(ref, "ugbase"),
                        "-I" + os.path.join(ROOT, "include"), "-I" + src_dir,
                        os.path.join(src_dir, "ug4gb_bridge.cpp")], capture_output=True, text=True)
    if negative:
        assert r.returncode != 0 and "ug4gb_disc_adjust_solution" in r.stderr
    else:
        assert r.returncode == 0, r.stderr[-4000:]
