"""
    CMDGCheckpoint

Exchange of checkpoints between libcmdg runs (`cmdg.checkpoint`, a raw
container: magic `CMDGCKP1`, a little-endian UInt64 header length, a JSON
header, then column-major arrays at 64-byte offsets) and ClimateMachine.jl
runs (`write_checkpoint` / `read_checkpoint`, JLD2 files holding `h_Q`,
`h_aux` and `t`, src/Driver/Checkpoint/Checkpoint.jl:21-127).

The state `h_Q` and the time `t` carry over as they are.  The auxiliary
state does not: the library stores only its reference state
(rho_ref, rhoe_ref, p_ref), the reference stores the whole aux of its
model, so each direction takes `h_aux` from the model that will restart:

    # a libcmdg checkpoint -> a JLD2 checkpoint a reference run restarts from
    cmdg_to_jld2("bubble_checkpoint_mpirank0000_num0003.cmdg", dg, "out", "bubble", 0, 3)
    # a reference checkpoint -> a libcmdg checkpoint
    jld2_to_cmdg("out", "bubble", 0, 3, "bubble_checkpoint_mpirank0000_num0003.cmdg"; h_aux = ref_state)

Not exercised in this repository's tests (no Julia here); the container's
layout is exercised from Python in tests/test_checkpoint_cpu.py.
"""
module CMDGCheckpoint

using JLD2
using JSON
using Printf

export read_cmdg, write_cmdg, cmdg_to_jld2, jld2_to_cmdg

const MAGIC = b"CMDGCKP1"
const ALIGN = 64
const DTYPES = Dict("<f8" => Float64, "<f4" => Float32)

"""
    read_cmdg(path) -> (arrays::Dict{String, Array}, header::Dict)

Every array record of a libcmdg checkpoint, in its Julia (column-major)
shape, and the JSON header (`"t"`, `"name"`, `"rank"`, `"num"`, ...).
"""
function read_cmdg(path::AbstractString)
    open(path, "r") do io
        read(io, 8) == MAGIC || error("$path is not a libcmdg checkpoint")
        hlen = ltoh(read(io, UInt64))
        header = JSON.parse(String(read(io, hlen)))
        arrays = Dict{String, Array}()
        for (name, rec) in header["arrays"]
            T = DTYPES[rec["dtype"]]
            A = Array{T}(undef, Tuple(Int.(rec["shape"]))...)
            seek(io, rec["offset"])
            read!(io, A)
            arrays[name] = A
        end
        return arrays, header
    end
end

"""
    write_cmdg(path, h_Q, h_aux, t; name = "", rank = 0, num = 0)

A libcmdg checkpoint with the FP64 state `h_Q` (Np, nstate, nelem), the
auxiliary record `h_aux` (Np, 3, nelem: rho_ref, rhoe_ref, p_ref) and `t`.
"""
function write_cmdg(path::AbstractString, h_Q::Array{Float64, 3}, h_aux::Array{Float64, 3}, t::Real;
                    name = "", rank = 0, num = 0)
    recs = [("h_Q", h_Q), ("h_aux", h_aux)]
    meta = Dict{String, Any}()
    # the arrays start after the header, each on a 64-byte boundary; the
    # header length depends on the offsets, so settle them by iteration
    offset0 = 0
    for _ in 1:4
        off = offset0
        for (nm, A) in recs
            off = cld(off, ALIGN) * ALIGN
            meta[nm] = Dict("dtype" => "<f8", "shape" => collect(size(A)), "offset" => off,
                            "nbytes" => sizeof(A))
            off += sizeof(A)
        end
        header = JSON.json(Dict("format" => "cmdg-checkpoint", "version" => 1, "t" => Float64(t),
                                "name" => name, "rank" => rank, "num" => num,
                                "arrays" => meta, "aux_fields" => ["rho_ref", "rhoe_ref", "p_ref"]))
        start = cld(16 + sizeof(header), ALIGN) * ALIGN
        if start == offset0
            open(path, "w") do io
                write(io, MAGIC)
                write(io, htol(UInt64(sizeof(header))))
                write(io, header)
                for (nm, A) in recs
                    write(io, zeros(UInt8, meta[nm]["offset"] - position(io)))
                    write(io, A)
                end
            end
            return path
        end
        offset0 = start
    end
    error("checkpoint header did not settle")
end

checkpoint_name(dir, name, rank, num) =
    joinpath(dir, @sprintf("%s_checkpoint_mpirank%04d_num%04d.jld2", replace(name, " " => "_"), rank, num))

"""
    cmdg_to_jld2(path, dg, checkpoint_dir, name, rank, num)

Writes the JLD2 checkpoint `read_checkpoint(checkpoint_dir, name, ..., num)`
of the reference loads: `h_Q` and `t` from the libcmdg checkpoint at `path`,
`h_aux` from the reference model `dg` that will restart
(`dg.state_auxiliary.realdata`).
"""
function cmdg_to_jld2(path, dg, checkpoint_dir, name, rank, num)
    arrays, header = read_cmdg(path)
    h_Q = arrays["h_Q"]
    h_aux = Array(dg.state_auxiliary.realdata)
    t = header["t"]
    cfull = checkpoint_name(checkpoint_dir, name, rank, num)
    @save cfull h_Q h_aux t
    return cfull
end

"""
    jld2_to_cmdg(checkpoint_dir, name, rank, num, path; h_aux)

A libcmdg checkpoint of the reference's JLD2 checkpoint: `h_Q` and `t`
from it, `h_aux` the library model's reference state (Np, 3, nelem), e.g.
from `cmdg_model_reference_state`.
"""
function jld2_to_cmdg(checkpoint_dir, name, rank, num, path; h_aux::Array{Float64, 3})
    cfull = checkpoint_name(checkpoint_dir, name, rank, num)
    @load cfull h_Q t
    return write_cmdg(path, Array{Float64}(h_Q), h_aux, t; name = name, rank = rank, num = num)
end

end # module
