"""The Fortran-subset translator that runs the reference's routines for the
golden vectors (`tests/golden/fortran_subset.py`), checked on a small module
written for this test: 1-based element and section access, column-major
array constructors and RESHAPE, integer division, do loops with steps and
empty ranges, block / one-line if with else-if, do concurrent, subroutine
calls with copy-out of intent(out) / intent(inout) arguments (whole
variables, elements and sections), functions returning arrays, complex
literals and kinds, parameters, and the preprocessor's serial branch; and
its emulation of unformatted I/O (stream, direct and sequential access,
either byte order)."""
import numpy as np

from tests.golden import fortran_subset as fs

SRC = """
module m_consts
   implicit none
   integer, parameter :: WP = 8
   real(kind=WP), parameter :: HALF = 0.5_WP
   complex(kind=WP), dimension(2, 2), parameter :: J2 = RESHAPE(source=[ &
        (1.0_WP, 0.0_WP), (0.0_WP, 2.0_WP), &
        (3.0_WP, 0.0_WP), (0.0_WP, -1.0_WP)], shape=[2, 2])
end module m_consts

module m_test
   use m_consts, only: WP, HALF, J2
   implicit none
contains
   pure subroutine scale2(out, a, k)
      real(kind=WP), dimension(:), intent(in) :: a
      real(kind=WP), dimension(size(a)), intent(out) :: out
      integer, intent(in) :: k
      out = a * k
   end subroutine scale2

   subroutine bump(x, n)
      integer, intent(inout) :: x
      integer, intent(in) :: n
      x = x + n
   end subroutine bump

   pure function rowsum(m, nr, nc) result(r)
      integer, intent(in) :: nr, nc
      real(kind=WP), dimension(nr, nc), intent(in) :: m
      real(kind=WP), dimension(nr) :: r
      integer :: i, j
      r = 0.0
      do i = 1, nr
         do j = nc, 1, -1
            r(i) = r(i) + m(i, j)
         end do
      end do
   end function rowsum

   function classify(v) result(c)
      integer, intent(in) :: v
      integer :: c
      if (v < 0) then
         c = -1
      else if (v == 0) then
         c = 0
      else
         c = 1
      end if
      if (v > 100) c = 2
   end function classify

   subroutine demo(res, cres, idiv, cnt, sec, conc)
      real(kind=WP), intent(out) :: res
      complex(kind=WP), intent(out) :: cres
      integer, intent(out) :: idiv, cnt
      real(kind=WP), dimension(4), intent(out) :: sec
      integer, intent(out) :: conc
      real(kind=WP), dimension(2, 3) :: m
      real(kind=WP), dimension(2) :: rs
      integer, dimension(3) :: iv
      integer :: k, a, b
      m = RESHAPE(source=[1.0_WP, 2.0_WP, 3.0_WP, 4.0_WP, 5.0_WP, 6.0_WP], shape=[2, 3])
      rs = rowsum(m, 2, 3)
      res = rs(1) * 10.0_WP + rs(2)
      cres = J2(2, 1) * J2(1, 2) + CONJG(J2(2, 2)) * HALF
      idiv = (7 / 2) * 100 + (-7 / 2)
      cnt = 0
      do k = 5, 4
         cnt = cnt + 1000
      end do
      do k = 1, 10, 3
         call bump(cnt, k)
      end do
      iv = (/1, 2, 3/)
      call bump(iv(2), 40)
      cnt = cnt + iv(2) + classify(-3) + classify(0) * 7 + classify(5) * 11 + classify(500) * 13
      sec = 0.0
      call scale2(sec(2:3), m(1, 2:3), 2)
#ifdef NEVER
      sec(1) = 99.0
#else
      sec(4) = 7.0
#endif
      conc = 0
      do concurrent(a=1:2, b=1:3)
         conc = conc + a * b
      end do
   end subroutine demo
end module m_test
"""


def test_translated_module_runs_as_fortran():
    tr = fs.Translator()
    tr.add_source(SRC)
    ns = tr.build()
    res, cres, idiv, cnt, sec, conc = ns["demo"](0.0, 0j, 0, 0, np.zeros(4), 0)
    # m = [[1,3,5],[2,4,6]] column-major: row sums 9 and 12
    assert res == 9 * 10 + 12
    # J2 column-major: J2(1,1)=1, J2(2,1)=2i, J2(1,2)=3, J2(2,2)=-i
    assert cres == (2j) * 3 + np.conj(-1j) * 0.5
    # integer division truncates towards zero
    assert idiv == 3 * 100 - 3
    # empty loop, steps 1,4,7,10, element copy-out, one-line and block if
    assert cnt == (1 + 4 + 7 + 10) + 42 + (-1) + 0 + 11 + 2 * 13
    # section arguments copied out: m(1, 2:3) = [3, 5] doubled into sec(2:3)
    assert list(sec) == [0.0, 6.0, 10.0, 7.0]
    assert conc == sum(a * b for a in (1, 2) for b in (1, 2, 3))


IO_SRC = """
module m_io
   implicit none
contains
   subroutine read_all(fstream, fdirect, fseq, n, ivals, x, rec2, seq2)
      character(len=*), intent(in) :: fstream, fdirect, fseq
      integer, intent(in) :: n
      integer, dimension(2), intent(out) :: ivals
      real(kind=8), intent(out) :: x
      complex(kind=8), dimension(n), intent(out) :: rec2
      real(kind=8), dimension(n, 2), intent(out) :: seq2
      integer :: k
      open (11, file=TRIM(fstream), form='unformatted', access='stream', status='old', convert='little_endian')
      read (11) ivals(1), ivals(2), x
      close (11)
      open (12, file=fdirect, form='unformatted', access='direct', recl=16 * n, convert='BIG_ENDIAN')
      read (12, rec=2) rec2
      close (12)
      open (13, file=fseq, form='unformatted', status='old', convert='BIG_ENDIAN')
      do k = 1, 2
         read (13) seq2(:, k)
      end do
      close (13)
   end subroutine read_all
end module m_io
"""


def test_translated_unformatted_io(tmp_path):
    """Stream (little-endian, mixed integer / real items), direct (big-endian
    fixed-length records, the second one read) and sequential (big-endian
    records framed by 4-byte lengths) access."""
    n = 3
    fs_ = tmp_path / "s.bin"
    fs_.write_bytes(np.array([7, -2], "<i4").tobytes() + np.array([2.5], "<f8").tobytes())
    fd = tmp_path / "d.bin"
    recs = np.arange(2 * n, dtype=np.float64).reshape(2, n) + 1j * 10
    fd.write_bytes(recs.astype(">c16").tobytes())
    fq = tmp_path / "q.bin"
    cols = [np.array([1.0, 2.0, 3.0]), np.array([4.0, 5.0, 6.0])]
    with open(fq, "wb") as fh:
        for c in cols:
            m = np.array([c.nbytes], ">i4").tobytes()
            fh.write(m + c.astype(">f8").tobytes() + m)
    tr = fs.Translator()
    tr.add_source(IO_SRC)
    ns = tr.build()
    ivals, x, rec2, seq2 = ns["read_all"](str(fs_), str(fd), str(fq), n, np.zeros(2, np.int64), 0.0,
                                          np.zeros(n, np.complex128), np.zeros((n, 2)))
    assert list(ivals) == [7, -2] and x == 2.5
    assert np.array_equal(rec2, recs[1])
    assert np.array_equal(seq2[:, 0], cols[0]) and np.array_equal(seq2[:, 1], cols[1])
