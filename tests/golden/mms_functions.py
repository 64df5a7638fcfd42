"""Generated by tests/golden/make_mms_functions.py: the manufactured solution
q(t, x, y, z) = (rho, U, V, W, E) of mms_solution.jl and its Navier-Stokes
source (gamma = cp_d / cv_d of the Earth constants, mu = 1/100)."""
import numpy


def q(t, x, y, z):
    c0 = numpy.pi*z
    c1 = numpy.sin(numpy.pi*x)*numpy.cos(numpy.pi*t)*numpy.cos(numpy.pi*y)
    c2 = c1*numpy.cos(c0)
    c3 = c2 + 3
    c4 = c2*c3
    return (c3, c4, c4, c1*c3*numpy.sin(c0), c2 + 100,)


def source(t, x, y, z):
    c0 = numpy.pi*z
    c1 = numpy.cos(c0)
    c2 = numpy.pi*c1
    c3 = numpy.pi*t
    c4 = numpy.sin(c3)
    c5 = numpy.pi*y
    c6 = numpy.cos(c5)
    c7 = numpy.pi*x
    c8 = numpy.sin(c7)
    c9 = c6*c8
    c10 = c4*c9
    c11 = c10*c2
    c12 = numpy.cos(c3)
    c13 = c12**2
    c14 = c6**2
    c15 = c13*c14
    c16 = numpy.sin(c0)
    c17 = c16**2
    c18 = c8**2
    c19 = numpy.pi*c18
    c20 = c17*c19
    c21 = c15*c20
    c22 = c1**2
    c23 = c19*c22
    c24 = numpy.sin(c5)
    c25 = c13*c24*c6
    c26 = c23*c25
    c27 = numpy.cos(c7)
    c28 = c1*c12
    c29 = c28*c9
    c30 = c29 + 3
    c31 = c24*c8
    c32 = numpy.pi*c31
    c33 = c19*c30
    c34 = c1**3
    c35 = c12**3
    c36 = c6**3
    c37 = c35*c36
    c38 = c27*c37
    c39 = c30**2
    c40 = c15*c39
    c41 = numpy.pi*c27
    c42 = c40*c41*c8
    c43 = 2*c30
    c44 = 2*c29
    c45 = c44 + 6
    c46 = 0.4/c45
    c47 = c46*(c1*c20*c38*c43 + 2*c17*c42 + 4*c22*c42 + 4*c33*c34*c38)
    c48 = numpy.pi**2
    c49 = (1/300)*c48
    c50 = c27*c6
    c51 = c45**(-2.0)
    c52 = c18*c40
    c53 = c17*c52 + 2*c22*c52
    c54 = c8**3
    c55 = numpy.pi*c54
    c56 = c14*c24*c35
    c57 = c55*c56
    c58 = c34*c57
    c59 = c17*c2*c54
    c60 = c14*c4
    c61 = -1/300*c1*c12*c24*c27*c48 - 1/30*c1*c12*c48*c6*c8 + c11*c30 + c12*c23*c60 - numpy.pi*c13*c14*c18*c22*c30 - 2*numpy.pi*c13*c14*c22*c27*c30*c8 - numpy.pi*c18*c27*c34*c35*c36 + c21*c30 + c26*c43 + c37*c59 + c58
    c62 = 4*c30
    c63 = 2*c25
    c64 = c28*c32
    c65 = 0.8*c51*c53
    c66 = c46*(-c20*c39*c63 - 4*c26*c39 - c43*c56*c59 - c58*c62) + c64*c65
    c67 = c37*c55
    c68 = c16**3*c67
    c69 = c12*c16
    c70 = c69*c9
    c71 = numpy.pi*c70
    c72 = c16*c22
    c73 = c16*c19
    c74 = c46*(-2*c1*c40*c73 - c43*c68 - c62*c67*c72) + c65*c71
    c75 = (1/100)*numpy.pi*c1*c12*c27*c6 - 1/100*c64
    c76 = c41*c6
    c77 = c28*c76
    c78 = (1/100)*c71
    c79 = (1/100)*numpy.pi*c12*c16*c27*c6 - c78
    c80 = -1/100*c32*c69 - c78
    c81 = (1/100)*c48
    c82 = c31*c81
    c83 = c70*c81
    c84 = c29*c81
    c85 = c24*c27
    c86 = (1/150)*c64
    c87 = numpy.pi*c29
    c88 = (1/150)*c87
    c89 = (1/150)*c77
    c90 = (1/150)*c48
    c91 = (1/75)*c48
    c92 = c28*c90
    c93 = c29*c91
    c94 = 1.4*c29 - c46*c53 + 140.0
    c95 = 1.4*c28
    return (numpy.pi*c1*c12*c27*c30*c6 + numpy.pi*c1*c12*c30*c6*c8 - c11 + numpy.pi*c13*c14*c22*c27*c8 - c21 - c26 - c28*c30*c32, 0.8*numpy.pi*c1*c12*c27*c51*c53*c6 + 0.4*numpy.pi*c1*c12*c27*c6 - c28*c49*c50 - c47 - c61, (1/300)*c1*c12*c24*c48*c8 - 0.4*c28*c32 - c61 - c66, 2*numpy.pi*c1*c13*c14*c16*c18*c30 + 2*numpy.pi*c1*c13*c14*c16*c27*c30*c8 - c1*c16*c33*c63 - numpy.pi*c10*c16*c30 + (1/300)*c12*c16*c27*c48*c6 + (1/30)*c12*c16*c48*c6*c8 + numpy.pi*c16*c18*c22*c27*c35*c36 - c28*c60*c73 - c31*c49*c69 - c57*c72 - c68 - 0.4*c71 - c74, numpy.pi*c1*c12*c24*c75*c8 + numpy.pi*c1*c12*c24*c8*(-1/75*c64 - c88 - c89) + numpy.pi*c1*c12*c27*c6*c94 + numpy.pi*c1*c12*c6*c8*c94 + c1*c12*c6*c8*(-c32*c95 - c66) + c1*c12*c6*c8*(-c47 + c65*c77 + c76*c95) - c11 + numpy.pi*c12*c16*c24*c8*c80 + numpy.pi*c12*c16*c6*c79*c8 + numpy.pi*c12*c16*c6*c8*c80 + c12*c16*c6*c8*(-1.4*c71 - c74) - c29*(-c28*c82 - c84) - c29*((1/100)*c1*c12*c27*c48*c6 - c84) - c29*(c31*c92 + c85*c92 - c93) - c29*((1/150)*c1*c12*c24*c27*c48 - c50*c92 - c93) - c44*(-c28*c81*c85 - c84) - c64*c94 - c69*c76*c79 - c70*(c69*c82 - c83) - c70*(-c50*c69*c81 - c83) - c70*((1/150)*c12*c16*c27*c48*c6 - c31*c69*c90 - c70*c91) - c75*c77 - c77*((1/75)*c77 + c86 - c88) - c87*(c86 + (1/75)*c87 - c89),)
