"""The Fortran-subset translator that runs the reference for the golden fixtures
(tests/golden/fortran_subset.py), checked on small programs written here: the
number semantics gfortran gives (integer division and mod, single-precision
literals and arithmetic, small integer powers), loops with negative strides,
pass by reference of scalars, array elements and sections, derived-type
records and their copies, module parameters and the one-rank MPI exchange."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import fortran_subset as fs  # noqa: E402

SRC = """
module m
    implicit none
    integer,parameter::n=4, nn=n*2
    real*8::x8
    type Rec
        integer::k
        real*8,dimension(1:3)::p
    end type
    type(Rec),dimension(1:n)::recs
    integer,dimension(:,:),allocatable::grid
endmodule
!---------------------------------------
subroutine divs(a,b,q,r)
use m
implicit none
    integer::a,b,q,r
    q = a/b
    r = mod(a,b)
return
endsubroutine
subroutine lits(y4,y8,z,w)
implicit none
    real*8::y4,y8,z,w
    y4 = 0.1
    y8 = 0.1d0
    z = 0.1*3.0
    w = 0.1*3d0 ! mixed: promoted
endsubroutine
subroutine powers(x,y2,y3,z3,zi)
implicit none
    real*8::x,y2,y3,z3,zi
    y2 = x**2; y3 = x**3
    z3 = 1.1**3
    zi = 16777217*1.0
endsubroutine
subroutine loops(s)
implicit none
    integer::s,i
    s = 0
    do i=10,1,-3
        s = s*100 + i
    enddo
endsubroutine
subroutine byref(a,b)
implicit none
    real*8::a
    real*8,dimension(1:3)::b
    a = a + 1d0
    b(2) = 7d0
endsubroutine
subroutine caller(out)
implicit none
    real*8::out(1:3)
    real*8::t
    t = 1d0
    call byref(t,out)
    out(1) = t
    call byref(out(3),out)
endsubroutine
subroutine records()
use m
implicit none
    recs(2)%k = 5
    recs(2)%p(:) = 0d0
    recs(2)%p(1) = 1.5d0
    recs(3) = recs(2)
    recs(2)%p(1) = -1d0
endsubroutine
subroutine sections(lo,hi)
use m
implicit none
    integer::lo,hi,i,j
    allocate(grid(lo:hi,0:2))
    grid(:,:) = 0
    grid(lo:lo+1,1) = 3
    do j=0,2
    do i=lo,hi
        if (i==hi.and.j==2) grid(i,j) = nn
    enddo
    enddo
endsubroutine
subroutine readfile(a,n)
implicit none
    integer::n,i
    real*8::a(1:3,1:2)
    character(len=20)::name
    name = "  pts.dat"
    open(10,file=adjustl(trim(name)))
    read(10,*) n
    do i=1,n
        read(10,*) a(1,i), a(2,i), a(3,i)
    enddo
    close(10)
    open(11,file="log.txt",access="append")
    write(11,*) "ignored", n
    close(11)
endsubroutine
subroutine oob(k,x)
implicit none
    integer::k
    real*8::x,a(1:3)
    a(:) = 1d0
    x = a(k)
endsubroutine
subroutine ring(me,got,total)
implicit none
    integer::me,got,total,mine,st(MPI_STATUS_SIZE),ierr,nr
    nr = 3
    mine = 10*(me+1)
    call MPI_SENDRECV(mine,1,MPI_INTEGER,mod(me+1,nr),7,got,1,MPI_INTEGER,mod(me+nr-1,nr),7,MPI_COMM_WORLD,st,ierr)
    call MPI_REDUCE(mine,total,1,MPI_INTEGER,MPI_SUM,0,MPI_COMM_WORLD,ierr)
    call MPI_BCAST(total,1,MPI_INTEGER,0,MPI_COMM_WORLD,ierr)
    call MPI_BARRIER(MPI_COMM_WORLD,ierr)
endsubroutine
subroutine sendself(out)
implicit none
    integer::out(1:2),buf(1:2),st(MPI_STATUS_SIZE),ierr
    buf(1) = 5; buf(2) = &
        6
    call MPI_SENDRECV(buf,2,MPI_INTEGER,0,1,out,2,MPI_INTEGER,0,1,MPI_COMM_WORLD,st,ierr)
endsubroutine
"""


def build():
    T = fs.Translator([("t.F90", SRC)])
    T.build()
    return T, T.new_state()


def test_integer_division_and_mod_truncate_toward_zero():
    T, G = build()
    for a, b in ((-7, 2), (7, -2), (7, 2), (-7, -2), (6, 3)):
        r = T.call(G, "divs", a, b, 0, 0)
        q = int(a / b)
        assert r[2:] == (q, a - b * q)


def test_default_real_literals_are_single_precision():
    T, G = build()
    y4, y8, z, w = T.call(G, "lits", 0.0, 0.0, 0.0, 0.0)
    f = np.float32
    assert y4 == float(f(0.1)) and y8 == 0.1
    assert z == float(f(f(0.1) * f(3.0)))
    assert w == float(f(0.1)) * 3.0


def test_small_integer_powers_are_products():
    T, G = build()
    x = 1.0 / 3.0
    _, y2, y3, z3, zi = T.call(G, "powers", x, 0.0, 0.0, 0.0, 0.0)
    assert y2 == x * x and y3 == (x * x) * x
    f = np.float32
    assert z3 == float(f(f(f(1.1) * f(1.1)) * f(1.1)))  # every single-precision product rounded
    assert zi == float(f(16777217))  # the integer operand converted to single first


def test_loop_with_negative_stride():
    T, G = build()
    assert T.call(G, "loops", 0)[0] == 10070401


def test_scalars_and_elements_pass_by_reference():
    T, G = build()
    out = np.zeros(3)
    T.call(G, "caller", out)
    assert list(out) == [2.0, 7.0, 1.0]


def test_record_assignment_copies():
    T, G = build()
    T.call(G, "records")
    assert G.m_recs.a["k"][2] == 5 and G.m_recs.a["p"][2, 0] == 1.5
    assert G.m_recs.a["p"][1, 0] == -1.0


def test_allocatable_bounds_and_sections():
    T, G = build()
    T.call(G, "sections", -1, 2)
    g = G.m_grid
    assert g.a.shape == (4, 3) and (g.o0, g.o1) == (-1, 0)
    assert list(g.a[:, 1]) == [3, 3, 0, 0] and g.a[3, 2] == 8 and g.a.sum() == 14


def test_mpi_sendrecv_to_self():
    T, G = build()
    out = np.zeros(2, np.int32)
    T.call(G, "sendself", out)
    assert list(out) == [5, 6]


def test_single_precision_literal_rounding_is_from_the_decimal():
    # 0.1 and 2.08e-4 rounded once from the decimal agree with numpy's float32 parse
    for text in ("0.1", "2.08e-4", "3.1415926536", "0.0183", "8.33"):
        assert fs._dec_to_f32(text) == float(np.float32(text))


def test_list_directed_reads(tmp_path):
    (tmp_path / "pts.dat").write_text("2\n 0.1 -2.5e-3  7\n\n1d-3, 4.0 5\n")
    T = fs.Translator([("t.F90", SRC)])
    T.build()
    G = T.new_state(io_dir=str(tmp_path))
    a = np.zeros((3, 2), order="F")
    r = T.call(G, "readfile", a, 0)
    assert r[1] == 2
    assert a[:, 0].tolist() == [0.1, -2.5e-3, 7.0] and a[:, 1].tolist() == [1e-3, 4.0, 5.0]
    assert not (tmp_path / "log.txt").exists()


def test_bounds_checks():
    import pytest

    T = fs.Translator([("t.F90", SRC)], check_bounds=True)
    T.build()
    G = T.new_state()
    assert T.call(G, "oob", 3, 0.0)[1] == 1.0
    for k in (0, 4):
        with pytest.raises(IndexError):
            T.call(G, "oob", k, 0.0)
    T.call(G, "sections", -1, 2)  # sections inside their bounds pass


def test_ranks_as_threads():
    """Three ranks sharing a World: a ring exchange, a sum at the root and its
    broadcast."""
    import threading

    T = fs.Translator([("t.F90", SRC)])
    T.build()
    world = fs.World(3, timeout=30.0)
    out = [None] * 3

    def rank(r):
        G = T.new_state()
        G.world, G.rank = world, r
        out[r] = T.call(G, "ring", r, 0, 0)

    threads = [threading.Thread(target=rank, args=(r,)) for r in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert [o[1] for o in out] == [30, 10, 20]
    assert [o[2] for o in out] == [60, 60, 60]
