"""Checks of the Fortran-to-numpy translator that generates the reference golden vectors.

Each case is a small fixed-form program whose result a Fortran compiler fixes
by the language rules: integer division, single-precision literals, scalar
arguments by reference, sequence association of array arguments, WHERE
blocks, labelled DO loops, COMMON storage.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import fexec  # noqa: E402

SRC = """\
      subroutine arith (n, m, q, r, s)
      integer n, m, q
      real*8 r, s
      q = n / m
      r = 0.1
      s = 0.1d0
      return
      end

      subroutine incr (k)
      k = k + 1
      end

      subroutine caller (out)
      integer out
      j = 4
      call incr (j)
      call incr (j)
      out = j
      end

      subroutine fill (a, n)
      dimension a(n)
      do i = 1, n
         a(i) = dble(i)
      enddo
      end

      subroutine seqasc (b)
      dimension b(3,4)
      call fill (b(1,2), 6)
      end

      subroutine masked (x, y, n)
      dimension x(n), y(n)
      where (x .gt. 0.5d0)
         y = 2.0d0 * x
      elsewhere (x .lt. -0.5d0)
         y = -1.0d0
      elsewhere
         y = 0.0d0
      endwhere
      end

      subroutine labloop (n, total)
      integer n, total
      total = 0
      do 10 i = 1, n
         if (i .eq. 3) cycle
         total = total + i
 10   continue
      end

      subroutine setcom (v)
      common /blk/ cv, icnt
      cv = v
      icnt = icnt + 1
      end
"""


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    d = tmp_path_factory.mktemp("f")
    (d / "t.f").write_text(SRC)
    P = fexec.Program([d])
    P.load(d / "t.f")
    return P


def test_integer_division_and_literal_kinds(prog):
    q, r, s = prog.call("arith", 7, -2, 0, 0.0, 0.0)[2:]
    assert q == -3  # truncation toward zero
    assert r == float(np.float32(0.1)) and r != 0.1  # a default-real literal is single precision
    assert s == 0.1


def test_scalar_arguments_are_passed_by_reference(prog):
    assert prog.call("caller", 0) == (6,)


def test_sequence_association_of_an_element_actual(prog):
    b = np.zeros((3, 4), order="F")
    prog.call("seqasc", b)
    assert np.array_equal(b[:, 0], [0, 0, 0])
    assert np.array_equal(b[:, 1:3].reshape(-1, order="F"), np.arange(1, 7))
    assert np.array_equal(b[:, 3], [0, 0, 0])


def test_where_elsewhere_blocks(prog):
    x = np.array([1.0, -1.0, 0.0, 0.7])
    y = np.full(4, np.nan)
    prog.call("masked", x, y, 4)
    assert np.array_equal(y, [2.0, -1.0, 0.0, 1.4])


def test_labelled_do_with_cycle(prog):
    assert prog.call("labloop", 5, 0) == (5, 12)


def test_common_blocks_persist(prog):
    prog.call("setcom", 2.5)
    prog.call("setcom", 3.5)
    assert prog.G.cv == 3.5 and prog.G.icnt == 2
